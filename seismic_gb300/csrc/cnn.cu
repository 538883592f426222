// cnn.cu - the convolutional gradient preconditioner (no reference
// counterpart): a small stack of 3x3 convolutions (ReLU between layers)
// that maps the FWI gradient and the source illumination to a search
// direction, with training and inference on the GPU.
//
// Activations and gradients are BF16 in channel-group planes: the channel
// count is rounded up to 8 (zeros above the layer's own count) and group g
// of 8 channels is a plane [x][z][8] of the image (pixel p = x * nz + z), so
// element (p, c) sits at ((c / 8) * npix + p) * 8 + c % 8.  One GEMM tile is
// a 32 (z) x 4 (x) patch of 128 pixels; an 8-channel slice of it, shifted by
// a tap, is one tensor copy of 4 contiguous 512-byte rows (zero fill outside
// the image) that lands in shared memory as 128 rows of 16 bytes - exactly
// one K column of core matrices of the tensor cores' no-swizzle layout
// (umma.cuh).
//
// * Convolution (forward, and the input gradient with mirrored taps and
//   transposed weights): implicit GEMM D[pixel][n] = sum over (tap,
//   channel) on tcgen05 (M = 128 pixels, N = 16 or 32 output channels,
//   K = 9 Cs), persistent CTAs, two shared-memory stages fed by TMA one
//   tile ahead, the accumulator in tensor memory.  The epilogue fuses the
//   bias and the ReLU (hidden layers write BF16 activations only), or the
//   ReLU derivative of the layer input (input gradient), or writes the FP32
//   output of the last layer.
// * Weight gradient: dW[tap, ci][co] = sum_p a[p + off(tap)][ci] dz[p][co]
//   on tcgen05 with both operands MN-major (the same tensor copies; K runs
//   over pixels), M = 128 rows of (tap, ci) plus one row of ones that gives
//   the bias gradient, N = output channels; each persistent CTA
//   accumulates its pixels in tensor memory and writes one partial sum,
//   and the partials are added in CTA order (deterministic).
//
// FP32 master weights and Adam state; the BF16 GEMM copies of the weights
// are rewritten in the tensor cores' layout after every update.
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

constexpr int kMaxC = 32;                 // channels per layer
constexpr int kTZ = 32, kTX = 4;          // pixel patch of one GEMM tile
constexpr int kTile = kTZ * kTX;          // 128 pixels = GEMM M
constexpr int kChunk = kTile * 16;        // one 8-channel slice: 2048 bytes
constexpr int kThreads = 128;
constexpr int kWgradSlots = 10 * kMaxC * kMaxC;   // partial sums per CTA

int r8(int c) { return (c + 7) / 8 * 8; }
int r16(int c) { return (c + 15) / 16 * 16; }

__device__ __forceinline__ unsigned char *align1024(unsigned char *p) {
  const unsigned a = umma_su32(p);
  return p + ((1024u - (a & 1023u)) & 1023u);
}
__device__ __forceinline__ void cnn_expect_tx(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(umma_su32(bar)),
               "r"(bytes)
               : "memory");
}
// Tensor copy of the 8-channel slice of channel group cg at pixels
// z0..z0+31 x x0..x0+3 (global -> shared memory, on an mbarrier).  The map's
// innermost dimension is (z, channel) flattened, so its coordinate 8 z is
// a multiple of 16 bytes for every z.
__device__ __forceinline__ void cnn_tma3(void *dst, const CUtensorMap *map, int cg, int z, int x,
                                         unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(umma_su32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(8 * z), "r"(x), "r"(cg),
      "r"(umma_su32(bar))
      : "memory");
}
// Instruction descriptor with both operands MN-major (transposed).
__host__ __device__ constexpr uint32_t umma_idesc_bf16_mn(int M, int N) {
  return umma_idesc_bf16(M, N) | (1u << 15) | (1u << 16);
}

__device__ __forceinline__ unsigned pack_bf16(float lo, float hi) {
  const __nv_bfloat16 a = __float2bfloat16(lo), b = __float2bfloat16(hi);
  return (unsigned)__bfloat16_as_ushort(a) | ((unsigned)__bfloat16_as_ushort(b) << 16);
}

// ---------------------------------------------------------------------------
// Implicit-GEMM 3x3 convolution.
//   D[p][n] = sum_{tap, c} in[p + s * off(tap)][c] * W[n][tap * Cs + c]
// with s = +1 (forward) or -1 (input gradient) and zero padding outside
// the image.  W: NP x kp BF16 in the tensor cores' K-major layout.
// ---------------------------------------------------------------------------
enum { kFwdHidden = 0, kFwdLast = 1, kBwd = 2 };

struct ConvArgs {
  int Cs;                        // stored input channels (multiple of 8)
  int nz, nx;
  int kp;                        // GEMM K: 9 Cs rounded up to 16
  int ntiles, tiles_z;
  int mirror;
  const __nv_bfloat16 *W;
  const float *bias;             // forward: nout biases
  int nout;                      // output channels
  int cs_out;                    // stored output channels (BF16 outputs)
  float *out32;                  // kFwdLast: [p][nout]
  __nv_bfloat16 *out16;          // kFwdHidden, kBwd: cs_out / 8 channel-group planes
  const __nv_bfloat16 *mask;     // kBwd: layer input activations (cs_out / 8 planes)
  int *err;
};

size_t conv_smem_bytes(int NP, int kp) {
  const size_t wbytes = ((size_t)NP * kp * 2 + 1023) / 1024 * 1024;
  return 1024 + wbytes + 2 * (size_t)(kp / 8) * kChunk;
}

template <int NP, int MODE>
__global__ void __launch_bounds__(kThreads, 1)
    k_conv_tma(const __grid_constant__ CUtensorMap amap, const ConvArgs A) {
  extern __shared__ unsigned char cnn_smem[];
  __shared__ __align__(8) unsigned long long full[2], mdone;
  __shared__ unsigned tmem_base;
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int nch = A.kp / 8, nload = 9 * (A.Cs / 8);
  unsigned char *base = align1024(cnn_smem);
  unsigned char *sW = base;
  unsigned char *st0 = base + ((size_t)NP * A.kp * 2 + 1023) / 1024 * 1024;
  const size_t sbytes = (size_t)nch * kChunk;
  if (tid == 0) {
    umma_mbar_init(&full[0]);
    umma_mbar_init(&full[1]);
    umma_mbar_init(&mdone);
    abort_flag = 0;
  }
  if (warp == 0) umma_alloc(&tmem_base, 32);
  for (int q = tid; q < NP * A.kp / 8; q += kThreads)
    reinterpret_cast<uint4 *>(sW)[q] = reinterpret_cast<const uint4 *>(A.W)[q];
  // K padding (one chunk when 9 Cs / 8 is odd) stays zero in both stages.
  for (int c = nload; c < nch; ++c)
    for (int q = tid; q < kChunk / 16; q += kThreads) {
      reinterpret_cast<uint4 *>(st0 + (size_t)c * kChunk)[q] = make_uint4(0, 0, 0, 0);
      reinterpret_cast<uint4 *>(st0 + sbytes + (size_t)c * kChunk)[q] = make_uint4(0, 0, 0, 0);
    }
  umma_fence_smem();
  umma_fence_before();
  __syncthreads();
  umma_fence_after();
  const unsigned tmem = tmem_base;
  const int first = blockIdx.x, stride = gridDim.x;
  const int nmine = first < A.ntiles ? (A.ntiles - 1 - first) / stride + 1 : 0;
  int issued = 0, consumed = 0, committed = 0;   // thread 0's counters
  auto issue = [&](int i) {
    const int t = first + i * stride;
    const int z0 = (t % A.tiles_z) * kTZ, x0 = (t / A.tiles_z) * kTX;
    unsigned char *dst = st0 + (size_t)(i & 1) * sbytes;
    cnn_expect_tx(&full[i & 1], (unsigned)(nload * kChunk));
    const int sgn = A.mirror ? -1 : 1;
    for (int tap = 0; tap < 9; ++tap) {
      const int dz = sgn * (tap % 3 - 1), dx = sgn * (tap / 3 - 1);
      for (int cg = 0; cg < A.Cs / 8; ++cg)
        cnn_tma3(dst + (size_t)(tap * (A.Cs / 8) + cg) * kChunk, &amap, cg, z0 + dz, x0 + dx,
                 &full[i & 1]);
    }
  };
  if (tid == 0 && nmine > 0) {
    issue(0);
    issued = 1;
  }
  for (int i = 0; i < nmine; ++i) {
    if (tid == 0) {
      // Stage (i + 1) & 1 held tile i - 1, whose products were waited for.
      if (i + 1 < nmine) {
        issue(i + 1);
        issued = i + 2;
      }
      if (!umma_mbar_wait(&full[i & 1], (i >> 1) & 1)) {
        abort_flag = 1;
        atomicOr(A.err, 1);
      } else {
        consumed = i + 1;
        umma_fence_after();
        constexpr uint32_t idesc = umma_idesc_bf16(kTile, NP);
        const unsigned sa = umma_su32(st0 + (size_t)(i & 1) * sbytes), sb = umma_su32(sW);
        for (int ks = 0; ks < A.kp / 16; ++ks) {
          const uint64_t ad = umma_smem_desc(sa + ks * 2 * kChunk, kChunk, 128);
          const uint64_t bd = umma_smem_desc(sb + ks * 2 * (NP / 8) * 128, (NP / 8) * 128, 128);
          umma_bf16(tmem, ad, bd, idesc, ks > 0);
        }
        umma_commit(&mdone);
        committed = i + 1;
      }
    }
    __syncthreads();
    if (abort_flag) break;
    bool ok = umma_mbar_wait(&mdone, i & 1);
    ok = __all_sync(0xffffffffu, ok);
    if (!ok) {
      abort_flag = 1;
      atomicOr(A.err, 1);
    }
    umma_fence_after();
    if (ok) {
      float acc[NP];
      const unsigned ta = tmem + ((unsigned)(warp * 32) << 16);
      umma_ld16(ta, acc);
      if (NP == 32) umma_ld16(ta + 16, acc + 16);
      const int t = first + i * stride;
      const int z = (t % A.tiles_z) * kTZ + (tid % kTZ);
      const int x = (t / A.tiles_z) * kTX + tid / kTZ;
      if (z < A.nz && x < A.nx) {
        const size_t p = (size_t)x * A.nz + z, npix = (size_t)A.nz * A.nx;
        if (MODE == kFwdLast) {
#pragma unroll
          for (int n = 0; n < NP; ++n)
            if (n < A.nout) A.out32[p * A.nout + n] = acc[n] + A.bias[n];
        } else {
#pragma unroll
          for (int c0 = 0; c0 < NP; c0 += 8) {
            if (c0 >= A.cs_out) break;
            float v[8];
            if (MODE == kFwdHidden) {
#pragma unroll
              for (int j = 0; j < 8; ++j)
                v[j] = c0 + j < A.nout ? fmaxf(acc[c0 + j] + A.bias[c0 + j], 0.f) : 0.f;
            } else {
              const uint4 mk =
                  *reinterpret_cast<const uint4 *>(A.mask + ((size_t)(c0 / 8) * npix + p) * 8);
              const unsigned mw[4] = {mk.x, mk.y, mk.z, mk.w};
#pragma unroll
              for (int j = 0; j < 8; ++j) {
                const unsigned short bits = (unsigned short)(mw[j >> 1] >> (16 * (j & 1)));
                const bool pos = __bfloat162float(__ushort_as_bfloat16(bits)) > 0.f;
                v[j] = (c0 + j < A.nout && pos) ? acc[c0 + j] : 0.f;
              }
            }
            *reinterpret_cast<uint4 *>(A.out16 + ((size_t)(c0 / 8) * npix + p) * 8) =
                make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]),
                           pack_bf16(v[6], v[7]));
          }
        }
      }
    }
    umma_fence_before();
    __syncthreads();
    if (abort_flag) break;
  }
  // After a give-up: wait (bounded) for this CTA's copies and products in
  // flight before the tensor memory and the CTA go away.
  if (tid == 0) {
    for (int j = consumed; j < issued; ++j) umma_mbar_wait(&full[j & 1], (j >> 1) & 1);
    if (committed > 0) umma_mbar_wait(&mdone, (committed - 1) & 1);
  }
  umma_fence_before();
  __syncthreads();
  umma_fence_after();
  if (warp == 0) umma_dealloc(tmem, 32);
}

// ---------------------------------------------------------------------------
// Weight and bias gradient of one layer on the tensor cores.
//   D[m][co] = sum_p A[m][p] * dz[p][co],  m = tap * Csi + ci  (A[m][p] =
//   a[p + off(tap)][ci]),  m = 9 Csi: a row of ones (bias gradient).
// Both operands MN-major: each 8-channel slice copied by TMA is one MN
// group of 8 rows x 128 pixels (core matrices 128 bytes apart along K, MN
// groups one 2048-byte slice apart).
// Stage layout: 9 Csi / 8 activation groups, the ones group, Cso / 8
// gradient groups, 2048 bytes each.  The M = 128 slices beyond the real
// rows read whatever shared memory follows (rows that are never stored).
// ---------------------------------------------------------------------------
struct WgradArgs {
  int Csi, Cin, Cso, Cout;
  int nz, nx, ntiles, tiles_z;
  int nmma;                      // M = 128 slices: ceil((9 Csi + 8) / 128)
  size_t stage_bytes;
  float *part;                   // [cta][10][kMaxC][kMaxC]
  int *err;
};

size_t wgrad_stage_bytes(int Csi, int Cso) {
  return (size_t)(9 * Csi / 8 + 1 + Cso / 8) * kChunk;
}
size_t wgrad_smem_bytes(int Csi, int Cso, int NPO) {
  const size_t sb = wgrad_stage_bytes(Csi, Cso);
  const int nmma = (9 * Csi + 8 + 127) / 128;
  const size_t reach = std::max({sb, (size_t)nmma * 16 * kChunk,
                                 (size_t)(9 * Csi / 8 + 1 + NPO / 8) * kChunk});
  return 1024 + sb + reach;
}

template <int NPO>
__global__ void __launch_bounds__(kThreads, 1)
    k_wgrad_umma(const __grid_constant__ CUtensorMap amap, const __grid_constant__ CUtensorMap dmap,
                 const WgradArgs A) {
  extern __shared__ unsigned char cnn_smem[];
  __shared__ __align__(8) unsigned long long full[2], mdone[2];
  __shared__ unsigned tmem_base;
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int G = 9 * A.Csi / 8;
  unsigned char *st0 = align1024(cnn_smem);
  if (tid == 0) {
    umma_mbar_init(&full[0]);
    umma_mbar_init(&full[1]);
    umma_mbar_init(&mdone[0]);
    umma_mbar_init(&mdone[1]);
    abort_flag = 0;
  }
  if (warp == 0) umma_alloc(&tmem_base, 128);
  // The ones group of both stages (BF16 1.0 = 0x3f80).
  for (int q = tid; q < kChunk / 16; q += kThreads) {
    const uint4 one = make_uint4(0x3f803f80u, 0x3f803f80u, 0x3f803f80u, 0x3f803f80u);
    reinterpret_cast<uint4 *>(st0 + (size_t)G * kChunk)[q] = one;
    reinterpret_cast<uint4 *>(st0 + A.stage_bytes + (size_t)G * kChunk)[q] = one;
  }
  umma_fence_smem();
  umma_fence_before();
  __syncthreads();
  umma_fence_after();
  const unsigned tmem = tmem_base;
  const int first = blockIdx.x, stride = gridDim.x;
  const int nmine = first < A.ntiles ? (A.ntiles - 1 - first) / stride + 1 : 0;
  const unsigned txb = (unsigned)((G + A.Cso / 8) * kChunk);
  auto issue = [&](int i) {
    const int t = first + i * stride;
    const int z0 = (t % A.tiles_z) * kTZ, x0 = (t / A.tiles_z) * kTX;
    unsigned char *dst = st0 + (size_t)(i & 1) * A.stage_bytes;
    cnn_expect_tx(&full[i & 1], txb);
    for (int tap = 0; tap < 9; ++tap) {
      const int dz = tap % 3 - 1, dx = tap / 3 - 1;
      for (int cg = 0; cg < A.Csi / 8; ++cg)
        cnn_tma3(dst + (size_t)(tap * (A.Csi / 8) + cg) * kChunk, &amap, cg, z0 + dz, x0 + dx,
                 &full[i & 1]);
    }
    for (int cg = 0; cg < A.Cso / 8; ++cg)
      cnn_tma3(dst + (size_t)(G + 1 + cg) * kChunk, &dmap, cg, z0, x0, &full[i & 1]);
  };
  if (tid == 0) {
    int issued = 0, consumed = 0, committed = 0;
    bool ok = true;
    if (nmine > 0) {
      issue(0);
      issued = 1;
    }
    constexpr uint32_t idesc = umma_idesc_bf16_mn(kTile, NPO);
    for (int i = 0; i < nmine && ok; ++i) {
      if (i + 1 < nmine) {
        // Stage (i + 1) & 1 is free once tile i - 1's products are done.
        if (i >= 1) ok = umma_mbar_wait(&mdone[(i - 1) & 1], ((i - 1) >> 1) & 1);
        if (!ok) break;
        issue(i + 1);
        issued = i + 2;
      }
      ok = umma_mbar_wait(&full[i & 1], (i >> 1) & 1);
      if (!ok) break;
      consumed = i + 1;
      umma_fence_after();
      const unsigned sa = umma_su32(st0 + (size_t)(i & 1) * A.stage_bytes);
      const unsigned sb = sa + (unsigned)((G + 1) * kChunk);
      for (int ks = 0; ks < kTile / 16; ++ks)
        for (int j = 0; j < A.nmma; ++j) {
          // MN-major, no swizzle: the leading byte offset is the step between
          // 8-row core-matrix groups along K (128 bytes here), the stride
          // byte offset the step between 8-element groups along M / N (one
          // 2048-byte slice).
          const uint64_t ad = umma_smem_desc(sa + j * 16 * kChunk + ks * 256, 128, kChunk);
          const uint64_t bd = umma_smem_desc(sb + ks * 256, 128, kChunk);
          umma_bf16(tmem + j * NPO, ad, bd, idesc, i > 0 || ks > 0);
        }
      umma_commit(&mdone[i & 1]);
      committed = i + 1;
    }
    if (!ok) {
      abort_flag = 1;
      atomicOr(A.err, 1);
      for (int j = consumed; j < issued; ++j) umma_mbar_wait(&full[j & 1], (j >> 1) & 1);
    }
    // Products complete in order: the last commit covers them all.
    if (committed > 0 && !umma_mbar_wait(&mdone[(committed - 1) & 1], ((committed - 1) >> 1) & 1)) {
      abort_flag = 1;
      atomicOr(A.err, 1);
    }
  }
  umma_fence_before();
  __syncthreads();
  umma_fence_after();
  if (!abort_flag && nmine > 0) {
    float *P = A.part + (size_t)blockIdx.x * kWgradSlots;
    for (int j = 0; j < A.nmma; ++j) {
      float acc[NPO];
      const unsigned ta = tmem + ((unsigned)(warp * 32) << 16) + j * NPO;
      umma_ld16(ta, acc);
      if (NPO == 32) umma_ld16(ta + 16, acc + 16);
      const int m = j * kTile + tid;
      if (m < 9 * A.Csi) {
        const int tap = m / A.Csi, ci = m % A.Csi;
        if (ci < A.Cin)
#pragma unroll
          for (int co = 0; co < NPO; ++co)
            if (co < A.Cout) P[(size_t)tap * kMaxC * kMaxC + co * kMaxC + ci] = acc[co];
      } else if (m == 9 * A.Csi) {
#pragma unroll
        for (int co = 0; co < NPO; ++co)
          if (co < A.Cout) P[(size_t)9 * kMaxC * kMaxC + co * kMaxC] = acc[co];
      }
    }
  }
  umma_fence_before();
  __syncthreads();
  umma_fence_after();
  if (warp == 0) umma_dealloc(tmem, 128);
}

// Sums the per-CTA partials in CTA order into the layer's gradient buffer
// (FP32, [co][tap][ci] then bias[co]) - added to what it holds.
__global__ void k_wgrad_sum(const float *__restrict__ part, int nchunk, int Cout, int Cin,
                            float *__restrict__ gw) {
  const int tap = blockIdx.x, t = threadIdx.x;
  const int co = t / kMaxC, ci = t % kMaxC;
  if (co >= Cout || (tap == 9 ? ci != 0 : ci >= Cin)) return;
  float s = 0.f;
  for (int c = 0; c < nchunk; ++c) s += part[(size_t)c * kWgradSlots + tap * kMaxC * kMaxC + t];
  if (tap == 9) gw[(size_t)Cout * 9 * Cin + co] += s;
  else gw[((size_t)co * 9 + tap) * Cin + ci] += s;
}

// Planar FP32 channels (c, p) -> BF16 channel-group planes with Cs stored
// channels (q = (g * npix + p) * 8 + c % 8).
__global__ void k_pack_input(const float *__restrict__ in, int C, int Cs, int npix,
                             __nv_bfloat16 *__restrict__ out) {
  const long long n = (long long)Cs * npix;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(q / (8LL * npix)) * 8 + (int)(q % 8);
    const long long p = (q / 8) % npix;
    out[q] = __float2bfloat16(c < C ? in[(size_t)c * npix + p] : 0.f);
  }
}

// Mean-square loss of a one-channel output: the output gradient
// (out - target) / npix as BF16 in channel 0 of one 8-channel plane, and
// per-block FP64 partial sums of (out - target)^2.
__global__ void k_loss(const float *__restrict__ out, const float *__restrict__ tgt, int npix,
                       __nv_bfloat16 *__restrict__ db, double *__restrict__ part) {
  __shared__ double red[256];
  double s = 0.0;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
    const float e = out[p] - tgt[p];
    s += (double)e * (double)e;
    *reinterpret_cast<uint4 *>(db + (size_t)p * 8) = make_uint4(pack_bf16(e / (float)npix, 0.f), 0u, 0u, 0u);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// Adam on the FP32 master weights.
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

// BF16 GEMM copies of one layer's weights in the tensor cores' K-major
// layout: forward NPo x KPf, element (co, tap * Csi + ci); input gradient
// NPi x KPb, element (ci, tap * Cso + co).  Zero outside the layer.
__global__ void k_weights_bf16(const float *__restrict__ w, int Cout, int Cin, int Csi, int Cso,
                               int NPo, int KPf, int NPi, int KPb,
                               __nv_bfloat16 *__restrict__ wf, __nv_bfloat16 *__restrict__ wb) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < NPo * KPf; q += gridDim.x * blockDim.x) {
    const int n = q / KPf, k = q % KPf;
    const int tap = k / Csi, ci = k % Csi;
    float v = 0.f;
    if (n < Cout && tap < 9 && ci < Cin) v = w[((size_t)n * 9 + tap) * Cin + ci];
    wf[umma_off(n, k, NPo) >> 1] = __float2bfloat16(v);
  }
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < NPi * KPb; q += gridDim.x * blockDim.x) {
    const int n = q / KPb, k = q % KPb;
    const int tap = k / Cso, co = k % Cso;
    float v = 0.f;
    if (n < Cin && tap < 9 && co < Cout) v = w[((size_t)co * 9 + tap) * Cin + n];
    wb[umma_off(n, k, NPi) >> 1] = __float2bfloat16(v);
  }
}

int nblk(long long n) { return (int)std::min<long long>(4096, (n + 255) / 256); }

// BF16 tensor map over Cs / 8 channel-group planes: dimensions (8 nz: z
// and the 8 channels flattened, nx, Cs / 8), box 8 kTZ x kTX x 1 (kTX rows
// of 512 bytes), zero fill outside.
bool encode_act_map(CUtensorMap *m, const __nv_bfloat16 *base, int Cs, int nz, int nx) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)nz * 8, (cuuint64_t)nx, (cuuint64_t)Cs / 8};
  const cuuint64_t strides[2] = {(cuuint64_t)nz * 16, (cuuint64_t)nz * nx * 16};
  const cuuint32_t box[3] = {8 * kTZ, kTX, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16 *>(base), dims,
             strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int num_sms(int dev) {
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1)
    n = 1;
  return n;
}

template <class K>
cudaError_t launch_big(K kernel, int grid, size_t smem, cudaStream_t s, const CUtensorMap &m0,
                       const ConvArgs &a) {
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  kernel<<<grid, kThreads, smem, s>>>(m0, a);
  return cudaGetLastError();
}

// One convolution: input tensor (Cs channels) -> MODE's outputs.
cudaError_t launch_conv(int dev, int mode, int NP, const __nv_bfloat16 *in, int Cs, int nz, int nx,
                        ConvArgs a, cudaStream_t s) {
  CUtensorMap m;
  if (!encode_act_map(&m, in, Cs, nz, nx)) return cudaErrorInvalidValue;
  a.Cs = Cs;
  a.nz = nz;
  a.nx = nx;
  a.kp = r16(9 * Cs);
  a.tiles_z = (nz + kTZ - 1) / kTZ;
  a.ntiles = a.tiles_z * ((nx + kTX - 1) / kTX);
  const size_t smem = conv_smem_bytes(NP, a.kp);
  const int per_sm = std::max<int>(1, std::min<int>(4, (int)((227u * 1024u) / smem)));
  const int grid = std::min(a.ntiles, num_sms(dev) * per_sm);
  if (NP == 16) {
    if (mode == kFwdHidden) return launch_big(k_conv_tma<16, kFwdHidden>, grid, smem, s, m, a);
    if (mode == kFwdLast) return launch_big(k_conv_tma<16, kFwdLast>, grid, smem, s, m, a);
    return launch_big(k_conv_tma<16, kBwd>, grid, smem, s, m, a);
  }
  if (mode == kFwdHidden) return launch_big(k_conv_tma<32, kFwdHidden>, grid, smem, s, m, a);
  if (mode == kFwdLast) return launch_big(k_conv_tma<32, kFwdLast>, grid, smem, s, m, a);
  return launch_big(k_conv_tma<32, kBwd>, grid, smem, s, m, a);
}

// Weight-gradient partials of one layer; returns the number of partials.
cudaError_t launch_wgrad(int dev, const __nv_bfloat16 *a, int Cin, const __nv_bfloat16 *dz,
                         int Cout, int nz, int nx, float *part, int *err, cudaStream_t s,
                         int *nchunk) {
  WgradArgs w;
  w.Csi = r8(Cin);
  w.Cin = Cin;
  w.Cso = r8(Cout);
  w.Cout = Cout;
  w.nz = nz;
  w.nx = nx;
  w.tiles_z = (nz + kTZ - 1) / kTZ;
  w.ntiles = w.tiles_z * ((nx + kTX - 1) / kTX);
  w.nmma = (9 * w.Csi + 8 + kTile - 1) / kTile;
  w.stage_bytes = wgrad_stage_bytes(w.Csi, w.Cso);
  w.part = part;
  w.err = err;
  CUtensorMap ma, md;
  if (!encode_act_map(&ma, a, w.Csi, nz, nx) || !encode_act_map(&md, dz, w.Cso, nz, nx))
    return cudaErrorInvalidValue;
  const int NPO = r16(Cout);
  const size_t smem = wgrad_smem_bytes(w.Csi, w.Cso, NPO);
  const int grid = std::min(w.ntiles, num_sms(dev));
  *nchunk = grid;
  cudaError_t e;
  if (NPO == 16) {
    e = cudaFuncSetAttribute(k_wgrad_umma<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return e;
    k_wgrad_umma<16><<<grid, kThreads, smem, s>>>(ma, md, w);
  } else {
    e = cudaFuncSetAttribute(k_wgrad_umma<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return e;
    k_wgrad_umma<32><<<grid, kThreads, smem, s>>>(ma, md, w);
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
  std::vector<__nv_bfloat16 *> a;      // layer inputs, r8(ch[l]) / 8 channel-group planes
  __nv_bfloat16 *dz[2] = {nullptr, nullptr};   // gradients, up to r8(max ch) / 8 planes
  float *out32 = nullptr, *in32 = nullptr, *tgt = nullptr, *part = nullptr;
  double *lpart = nullptr;
  int *err = nullptr;
};

namespace {

int cnn_fail(sw_cnn *n, cudaError_t e, const char *what) {
  return cuda_fail(n ? n->ctx : nullptr, e, what);
}

void free_images(sw_cnn *n) {
  for (auto p : n->a) cudaFree(p);
  n->a.clear();
  cudaFree(n->dz[0]); cudaFree(n->dz[1]);
  cudaFree(n->out32); cudaFree(n->in32); cudaFree(n->tgt); cudaFree(n->part); cudaFree(n->lpart);
  n->dz[0] = n->dz[1] = nullptr;
  n->out32 = n->in32 = n->tgt = n->part = nullptr;
  n->lpart = nullptr;
  n->cap = 0;
}

int ensure_images(sw_cnn *n, size_t npix) {
  if (npix <= n->cap) return SW_OK;
  free_images(n);
  auto ck = [&](cudaError_t e) { return e == cudaSuccess; };
  bool ok = true;
  int cmax = 8;
  for (int c : n->ch) cmax = std::max(cmax, r8(c));
  n->a.assign(n->nl, nullptr);
  for (int l = 0; l < n->nl && ok; ++l)
    ok = ck(cudaMalloc(&n->a[l], npix * r8(n->ch[l]) * sizeof(__nv_bfloat16)));
  ok = ok && ck(cudaMalloc(&n->dz[0], npix * cmax * sizeof(__nv_bfloat16))) &&
       ck(cudaMalloc(&n->dz[1], npix * cmax * sizeof(__nv_bfloat16))) &&
       ck(cudaMalloc(&n->out32, npix * sizeof(float))) &&
       ck(cudaMalloc(&n->in32, npix * n->ch[0] * sizeof(float))) &&
       ck(cudaMalloc(&n->tgt, npix * sizeof(float))) &&
       ck(cudaMalloc(&n->part, (size_t)num_sms(n->ctx->device) * kWgradSlots * sizeof(float))) &&
       ck(cudaMalloc(&n->lpart, 1024 * sizeof(double)));
  if (!ok) {
    cudaGetLastError();
    free_images(n);
    return fail(n->ctx, SW_OOM_ADMISSION, "cnn image buffers");
  }
  n->cap = npix;
  return SW_OK;
}

// Runs one tensor-core kernel launch; with profiling on, brackets it with
// CUDA events on the context stream and adds its time, algorithmic bytes
// and FLOPs to the context's counters.
template <class L>
cudaError_t timed_launch(sw_cnn *n, uint64_t bytes, uint64_t flops, L launch) {
  sw_ctx *c = n->ctx;
  c->stats.launches_total++;
  if (!c->profiling) return launch();
  cudaEvent_t e0, e1;
  cudaError_t e = cudaEventCreate(&e0);
  if (e != cudaSuccess) return e;
  if ((e = cudaEventCreate(&e1)) != cudaSuccess) {
    cudaEventDestroy(e0);
    return e;
  }
  cudaEventRecord(e0, c->stream);
  e = launch();
  cudaEventRecord(e1, c->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e == cudaSuccess) {
    c->stats.cnn_conv_ms += ms;
    c->stats.cnn_conv_timed++;
    c->stats.cnn_conv_bytes += bytes;
    c->stats.cnn_conv_flops += flops;
  }
  return e;
}

int refresh_bf16(sw_cnn *n) {
  cudaStream_t s = n->ctx->stream;
  for (int l = 0; l < n->nl; ++l) {
    const int Cin = n->ch[l], Cout = n->ch[l + 1];
    k_weights_bf16<<<8, 256, 0, s>>>(n->w + n->woff[l], Cout, Cin, r8(Cin), r8(Cout), r16(Cout),
                                     r16(9 * r8(Cin)), r16(Cin), r16(9 * r8(Cout)), n->wf[l],
                                     n->wb[l]);
    n->ctx->stats.launches_total++;
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SW_OK : cnn_fail(n, e, "cnn weights");
}

// Forward pass of one image already packed into n->a[0]; output in n->out32.
int forward(sw_cnn *n, int nz, int nx) {
  cudaStream_t s = n->ctx->stream;
  const int dev = n->ctx->device;
  cudaError_t e;
  for (int l = 0; l < n->nl; ++l) {
    const int Cin = n->ch[l], Cout = n->ch[l + 1];
    const bool last = l + 1 == n->nl;
    ConvArgs a{};
    a.mirror = 0;
    a.W = n->wf[l];
    a.bias = n->w + n->woff[l] + (size_t)Cout * 9 * Cin;
    a.nout = Cout;
    a.cs_out = r8(Cout);
    a.out32 = last ? n->out32 : nullptr;
    a.out16 = last ? nullptr : n->a[l + 1];
    a.err = n->err;
    const uint64_t np = (uint64_t)nz * nx;
    const uint64_t bytes = np * r8(Cin) * 2 + (last ? np * Cout * 4 : np * r8(Cout) * 2);
    if ((e = timed_launch(n, bytes, 2 * np * Cout * 9 * Cin, [&] {
           return launch_conv(dev, last ? kFwdLast : kFwdHidden, r16(Cout), n->a[l], r8(Cin), nz,
                              nx, a, s);
         })) != cudaSuccess)
      return cnn_fail(n, e, "cnn conv");
  }
  return SW_OK;
}

int check_err(sw_cnn *n) {
  int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, n->err, sizeof(int), cudaMemcpyDeviceToHost, n->ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(n->ctx->stream);
  if (e != cudaSuccess) return cnn_fail(n, e, "cnn");
  if (h) {
    cudaMemsetAsync(n->err, 0, sizeof(int), n->ctx->stream);
    return fail(n->ctx, SW_TIMEOUT, "cnn: a tensor-core or tensor-copy wait gave up");
  }
  return SW_OK;
}

// Sum over the batch of the weight gradient into n->g (zeroed first); the
// batch-mean loss into *loss.
int gradient(sw_cnn *n, int nbatch, int nz, int nx, const float *in, const float *target,
             double *loss) {
  cudaStream_t s = n->ctx->stream;
  const int dev = n->ctx->device;
  const size_t npix = (size_t)nz * nx;
  int st = ensure_images(n, npix);
  if (st) return st;
  cudaError_t e;
  if ((e = cudaMemsetAsync(n->g, 0, n->nw * 4, s)) != cudaSuccess) return cnn_fail(n, e, "cnn");
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
    k_pack_input<<<nblk((long long)npix * r8(n->ch[0])), 256, 0, s>>>(
        n->in32, n->ch[0], r8(n->ch[0]), (int)npix, n->a[0]);
    n->ctx->stats.launches_total++;
    if ((st = forward(n, nz, nx))) return st;
    // d loss / d output (one channel), FP64 loss partials.
    int cur = 0;
    k_loss<<<lblocks, 256, 0, s>>>(n->out32, n->tgt, (int)npix, n->dz[cur], n->lpart);
    n->ctx->stats.launches_total++;
    for (int l = n->nl - 1; l >= 0; --l) {
      const int Cin = n->ch[l], Cout = n->ch[l + 1];
      int nchunk = 0;
      const uint64_t np = (uint64_t)npix;
      if ((e = timed_launch(n, np * (r8(Cin) + r8(Cout)) * 2, 2 * np * 9 * Cin * Cout, [&] {
             return launch_wgrad(dev, n->a[l], Cin, n->dz[cur], Cout, nz, nx, n->part, n->err, s,
                                 &nchunk);
           })) != cudaSuccess)
        return cnn_fail(n, e, "cnn wgrad");
      k_wgrad_sum<<<10, kMaxC * kMaxC, 0, s>>>(n->part, nchunk, Cout, Cin, n->g + n->woff[l]);
      n->ctx->stats.launches_total++;
      if (l == 0) break;
      // Input gradient: mirrored taps, transposed weights, then ReLU' of
      // the layer input, into the other gradient buffer.
      ConvArgs a{};
      a.mirror = 1;
      a.W = n->wb[l];
      a.bias = nullptr;
      a.nout = Cin;
      a.cs_out = r8(Cin);
      a.out16 = n->dz[cur ^ 1];
      a.mask = n->a[l];
      a.err = n->err;
      if ((e = timed_launch(n, np * (r8(Cout) + 2 * r8(Cin)) * 2, 2 * np * Cin * 9 * Cout, [&] {
             return launch_conv(dev, kBwd, r16(Cin), n->dz[cur], r8(Cout), nz, nx, a, s);
           })) != cudaSuccess)
        return cnn_fail(n, e, "cnn dgrad");
      cur ^= 1;
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
  if (loss) *loss = lsum / nbatch;
  return SW_OK;
}

}  // namespace

extern "C" {

int sw_cnn_create(sw_ctx *c, int nlayers, const int *channels, uint64_t seed, sw_cnn **out) {
  if (!c || !channels || !out || nlayers < 1 || nlayers > 16) return SW_BAD_PARAM;
  *out = nullptr;
  for (int l = 0; l <= nlayers; ++l)
    if (channels[l] < 1 || channels[l] > kMaxC)
      return fail(c, SW_BAD_PARAM, "cnn channels must be 1..32");
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
  for (int l = 0; l < nlayers && ok; ++l) {
    const int Cin = n->ch[l], Cout = n->ch[l + 1];
    ok = ck(cudaMalloc(&n->wf[l], (size_t)r16(Cout) * r16(9 * r8(Cin)) * 2)) &&
         ck(cudaMalloc(&n->wb[l], (size_t)r16(Cin) * r16(9 * r8(Cout)) * 2));
  }
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
  k_pack_input<<<nblk((long long)npix * r8(n->ch[0])), 256, 0, s>>>(n->in32, n->ch[0],
                                                                     r8(n->ch[0]), (int)npix,
                                                                     n->a[0]);
  n->ctx->stats.launches_total++;
  if ((st = forward(n, nz, nx))) return st;
  if ((e = cudaMemcpyAsync(out, n->out32, npix * 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return cnn_fail(n, e, "cnn output");
  return check_err(n);
}

int sw_cnn_gradient(sw_cnn *n, int nbatch, int nz, int nx, const float *in, const float *target,
                    float *grad, double *loss) {
  if (!n || !in || !target || !grad || nbatch < 1 || nz < 1 || nx < 1) return SW_BAD_PARAM;
  if (n->ch[n->nl] != 1) return fail(n->ctx, SW_BAD_PARAM, "cnn output must have one channel");
  cudaSetDevice(n->ctx->device);
  int st = gradient(n, nbatch, nz, nx, in, target, loss);
  if (st) return st;
  if ((st = check_err(n))) return st;
  std::vector<float> h(n->nw);
  if (cudaMemcpy(h.data(), n->g, n->nw * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return SW_CUDA_ERR;
  for (size_t q = 0; q < n->nw; ++q) grad[q] = h[q] / (float)nbatch;
  return SW_OK;
}

int sw_cnn_train_step(sw_cnn *n, int nbatch, int nz, int nx, const float *in,
                      const float *target, float lr, double *loss) {
  if (!n || !in || !target || nbatch < 1 || nz < 1 || nx < 1) return SW_BAD_PARAM;
  if (n->ch[n->nl] != 1) return fail(n->ctx, SW_BAD_PARAM, "cnn output must have one channel");
  cudaSetDevice(n->ctx->device);
  cudaStream_t s = n->ctx->stream;
  int st = gradient(n, nbatch, nz, nx, in, target, loss);
  if (st) return st;
  // Adam (b1 0.9, b2 0.999, eps 1e-8) on the batch-mean gradient.
  n->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)n->step), c2 = 1.f - std::pow(b2, (float)n->step);
  k_adam<<<(int)((n->nw + 255) / 256), 256, 0, s>>>(n->w, n->g, n->m, n->v, (int)n->nw, lr, b1, b2,
                                                    1e-8f, c1, c2, 1.f / (float)nbatch);
  n->ctx->stats.launches_total++;
  if ((st = refresh_bf16(n))) return st;
  return check_err(n);
}

}  // extern "C"
