// cnn.cu - the convolutional gradient preconditioner (no reference
// counterpart): a small stack of 3x3 convolutions (ReLU between layers)
// that maps the FWI gradient and the source illumination to a search
// direction, with training and inference on the GPU.
//
// Activations and gradients are BF16 in channel-group planes: the channel
// count is rounded up to 16 (zeros above the layer's own count) and group g
// of 8 channels is a plane [x][z][8] of the image (pixel p = x * nz + z), so
// element (p, c) sits at ((c / 8) * npix + p) * 8 + c % 8.  One GEMM tile is
// a 32 (z) x 4 (x) patch of 128 pixels; the 8-channel slice of a tap-shifted
// patch is 4 contiguous 512-byte rows that land in shared memory as 128 rows
// of 16 bytes - exactly one K column of core matrices of the tensor cores'
// no-swizzle layout (umma.cuh) - and one tensor copy fetches the slices of
// all channel groups of a tap (zero fill outside the image).
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
constexpr int kWgradSlots = 28 * kMaxC * kMaxC;   // partial sums per CTA (27 taps + bias)

int r16(int c);
// Stored channels of a tensor: a multiple of 16, so that one tap of a
// layer's input is a whole number of K = 16 steps.
int cstore(int c) { return (c + 15) / 16 * 16; }
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
// z..z+31 x x..x+3 of plane y (global -> shared memory, on an mbarrier).
// The map's innermost dimension is (z, channel) flattened, so its
// coordinate 8 z is a multiple of 16 bytes for every z.
__device__ __forceinline__ void cnn_tma4(void *dst, const CUtensorMap *map, int cg, int z, int x,
                                         int y, unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(umma_su32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(8 * z), "r"(x), "r"(y), "r"(cg),
      "r"(umma_su32(bar))
      : "memory");
}
// Offsets of tap t of a 3 x 3 (taps = 9) or 3 x 3 x 3 (taps = 27) kernel:
// t = 9 (dy + 1) + 3 (dx + 1) + (dz + 1).
__device__ __forceinline__ void tap_off(int t, int taps, int &dz, int &dx, int &dy) {
  dz = t % 3 - 1;
  dx = (t / 3) % 3 - 1;
  dy = taps == 27 ? t / 9 - 1 : 0;
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
// Warp roles of both kernels (192 threads): warps 0-3 read the tensor-memory
// accumulator (lane quadrant = warp) and run the epilogue, warp 4 issues
// the tensor copies into a ring of shared-memory stages, warp 5 issues the
// tensor-core instructions.  Every wait is bounded; a wait that gives up
// sets the error flag and the CTA's abort flag, and every role leaves its
// loop at its next wait.
// ---------------------------------------------------------------------------
constexpr int kEpiWarps = 4, kProducerWarp = 4, kMmaWarp = 5;
constexpr int kWsThreads = 192;

// Bounded wait that also gives up once another role has aborted.
__device__ __forceinline__ bool cnn_wait(unsigned long long *bar, unsigned parity,
                                         volatile int *abort_flag) {
  for (int it = 0; it < (1 << 22); ++it) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(umma_su32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
    if ((it & 63) == 63 && *abort_flag) return false;
  }
  return false;
}
__device__ __forceinline__ void cnn_arrive(unsigned long long *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(umma_su32(bar)) : "memory");
}
__device__ __forceinline__ void cnn_bar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(umma_su32(bar)), "r"(count)
               : "memory");
}

// ---------------------------------------------------------------------------
// Implicit-GEMM 3x3 (or 3x3x3) convolution.
//   D[p][n] = sum_{tap, c} in[p + s * off(tap)][c] * W[n][tap * Cs + c]
// with s = +1 (forward) or -1 (input gradient) and zero padding outside
// the image.  W: NP x kp BF16 in the tensor cores' K-major layout.  One
// ring stage holds one kernel row (a dz, and a dy in 3D): a single tensor
// copy of the patch shifted by dz and widened to 6 columns (x0 - 1 ..
// x0 + 4), every channel group.  In a plane of that copy ([6 x][32 z][8])
// the patch shifted by dx is the contiguous run of 128 rows from column
// dx + 1, so the three dx taps are three A operands of the same stage
// (3 Cs / 16 K = 16 steps).  Two accumulators in tensor memory let the
// products of the next tile run while the epilogue reads the last one.
// ---------------------------------------------------------------------------
enum { kFwdHidden = 0, kFwdLast = 1, kBwd = 2 };
constexpr int kMaxRing = 32;

struct ConvArgs {
  int Cs;                        // stored input channels (multiple of 16)
  int nz, nx, ny;
  int taps;                      // 9 (2D) or 27 (3D)
  int kp;                        // GEMM K: taps Cs
  int ntiles, tiles_z, tiles_x;
  int mirror;
  int ring;                      // shared-memory stages (<= kMaxRing)
  const __nv_bfloat16 *W;
  const float *bias;             // forward: nout biases
  int nout;                      // output channels
  int cs_out;                    // stored output channels (BF16 outputs)
  float *out32;                  // kFwdLast: [p][nout]
  __nv_bfloat16 *out16;          // kFwdHidden, kBwd: cs_out / 8 channel-group planes
  const __nv_bfloat16 *mask;     // kBwd: layer input activations (cs_out / 8 planes)
  int *err;
};

__host__ __device__ inline size_t conv_wbytes(int NP, int kp) { return ((size_t)NP * kp * 2 + 1023) / 1024 * 1024; }
constexpr int kConvCols = kTX + 2;                 // copy width: the patch and its x halo
constexpr int kConvPlane = kConvCols * kTZ * 16;   // bytes of one channel group in a stage
size_t conv_smem_bytes(int NP, int kp, int Cs, int ring) {
  return 1024 + conv_wbytes(NP, kp) + (size_t)ring * (Cs / 8) * kConvPlane;
}

template <int NP, int MODE>
__global__ void __launch_bounds__(kWsThreads, 1)
    k_conv_tma(const __grid_constant__ CUtensorMap amap, const ConvArgs A) {
  extern __shared__ unsigned char cnn_smem[];
  __shared__ __align__(8) unsigned long long full[kMaxRing], empty[kMaxRing];
  __shared__ __align__(8) unsigned long long acc_full[2], acc_empty[2];
  __shared__ unsigned tmem_base;
  __shared__ volatile int abort_flag;
  __shared__ volatile int mma_stages;             // stages the MMA warp has consumed
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nst = A.taps / 3;                     // ring stages (kernel rows) per tile
  const size_t sbytes = (size_t)(A.Cs / 8) * kConvPlane;   // one kernel row
  unsigned char *base = align1024(cnn_smem);
  unsigned char *sW = base;
  unsigned char *ring = base + conv_wbytes(NP, A.kp);
  if (tid == 0) {
    for (int q = 0; q < A.ring; ++q) {
      cnn_bar_init(&full[q], 1);
      cnn_bar_init(&empty[q], 1);
    }
    for (int q = 0; q < 2; ++q) {
      cnn_bar_init(&acc_full[q], 1);
      cnn_bar_init(&acc_empty[q], kEpiWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
    mma_stages = 0;
  }
  if (warp == kMmaWarp) umma_alloc(&tmem_base, 64);
  for (int q = tid; q < NP * A.kp / 8; q += kWsThreads)
    reinterpret_cast<uint4 *>(sW)[q] = reinterpret_cast<const uint4 *>(A.W)[q];
  umma_fence_smem();
  umma_fence_before();
  __syncthreads();
  umma_fence_after();
  const unsigned tmem = tmem_base;
  const int first = blockIdx.x, stride = gridDim.x;
  const int nmine = first < A.ntiles ? (A.ntiles - 1 - first) / stride + 1 : 0;
  if (warp == kProducerWarp) {
    if (lane == 0) {
      const int sgn = A.mirror ? -1 : 1;
      int q = 0;
      bool ok = true;
      for (int i = 0; i < nmine && ok; ++i) {
        const int t = first + i * stride;
        const int z0 = (t % A.tiles_z) * kTZ, x0 = ((t / A.tiles_z) % A.tiles_x) * kTX;
        const int y0 = t / (A.tiles_z * A.tiles_x);
        for (int k = 0; k < nst; ++k, ++q) {
          const int slot = q % A.ring;
          if (q >= A.ring && !(ok = cnn_wait(&empty[slot], ((q / A.ring) - 1) & 1, &abort_flag)))
            break;
          unsigned char *dst = ring + (size_t)slot * sbytes;
          cnn_expect_tx(&full[slot], (unsigned)sbytes);
          // Kernel row k: dz = k % 3 - 1, dy = k / 3 - 1 (3D).
          const int dz = k % 3 - 1, dy = A.taps == 27 ? k / 3 - 1 : 0;
          cnn_tma4(dst, &amap, 0, z0 + sgn * dz, x0 - 1, y0 + sgn * dy, &full[slot]);
        }
      }
      if (!ok) {
        abort_flag = 1;
        atomicOr(A.err, 1);
      }
      // After a give-up, copies the MMA warp did not consume complete
      // before the CTA leaves (at most one ring of them).
      if (abort_flag)
        for (int r = max(mma_stages, q - A.ring); r < q; ++r)
          umma_mbar_wait(&full[r % A.ring], (r / A.ring) & 1);
    }
  } else if (warp == kMmaWarp) {
    if (lane == 0) {
      constexpr uint32_t idesc = umma_idesc_bf16(kTile, NP);
      const unsigned sb = umma_su32(sW);
      int q = 0, committed = -1;
      bool ok = true;
      for (int i = 0; i < nmine && ok; ++i) {
        const int acc = i & 1;
        if (i >= 2 && !(ok = cnn_wait(&acc_empty[acc], ((i >> 1) - 1) & 1, &abort_flag))) break;
        umma_fence_after();
        const unsigned d = tmem + acc * NP;
        for (int k = 0; k < nst; ++k, ++q) {
          const int slot = q % A.ring;
          if (!(ok = cnn_wait(&full[slot], (q / A.ring) & 1, &abort_flag))) break;
          mma_stages = q + 1;
          umma_fence_after();
          const unsigned sa = umma_su32(ring + (size_t)slot * sbytes);
          const int dz = k % 3 - 1, dy = A.taps == 27 ? k / 3 - 1 : 0;
          for (int dx = -1; dx <= 1; ++dx) {
            // Tap of (dz, dx, dy); its A operand starts at column s dx + 1.
            const int t = 9 * (dy + 1) + 3 * (dx + 1) + (dz + 1) - (A.taps == 27 ? 0 : 9);
            const unsigned col = (unsigned)((A.mirror ? -dx : dx) + 1) * kTZ * 16;
            for (int h = 0; h < A.Cs / 16; ++h) {
              const int ks = t * (A.Cs / 16) + h;
              const uint64_t ad = umma_smem_desc(sa + h * 2 * kConvPlane + col, kConvPlane, 128);
              const uint64_t bd =
                  umma_smem_desc(sb + ks * 2 * (NP / 8) * 128, (NP / 8) * 128, 128);
              umma_bf16(d, ad, bd, idesc, k > 0 || dx > -1 || h > 0);
            }
          }
          umma_commit(&empty[slot]);
        }
        if (!ok) break;
        umma_commit(&acc_full[acc]);
        committed = i;
      }
      if (!ok) {
        abort_flag = 1;
        atomicOr(A.err, 1);
      }
      if (committed >= 0) umma_mbar_wait(&acc_full[committed & 1], (committed >> 1) & 1);
    }
  } else {
    // Epilogue: thread = accumulator lane = pixel row of the tile.
    for (int i = 0; i < nmine; ++i) {
      const int acc = i & 1;
      bool ok = cnn_wait(&acc_full[acc], (i >> 1) & 1, &abort_flag);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) {
        if (lane == 0) {
          abort_flag = 1;
          atomicOr(A.err, 1);
        }
        break;
      }
      umma_fence_after();
      float accv[NP];
      const unsigned ta = tmem + ((unsigned)(warp * 32) << 16) + acc * NP;
      umma_ld16(ta, accv);
      if (NP == 32) umma_ld16(ta + 16, accv + 16);
      umma_fence_before();
      __syncwarp();
      if (lane == 0) cnn_arrive(&acc_empty[acc]);
      const int t = first + i * stride;
      const int z = (t % A.tiles_z) * kTZ + (tid % kTZ);
      const int x = ((t / A.tiles_z) % A.tiles_x) * kTX + tid / kTZ;
      const int y = t / (A.tiles_z * A.tiles_x);
      if (z < A.nz && x < A.nx) {
        const size_t p = ((size_t)y * A.nx + x) * A.nz + z;
        const size_t npix = (size_t)A.nz * A.nx * A.ny;
        if (MODE == kFwdLast) {
#pragma unroll
          for (int n = 0; n < NP; ++n)
            if (n < A.nout) A.out32[p * A.nout + n] = accv[n] + A.bias[n];
        } else {
#pragma unroll
          for (int c0 = 0; c0 < NP; c0 += 8) {
            if (c0 >= A.cs_out) break;
            float v[8];
            if (MODE == kFwdHidden) {
#pragma unroll
              for (int j = 0; j < 8; ++j)
                v[j] = c0 + j < A.nout ? fmaxf(accv[c0 + j] + A.bias[c0 + j], 0.f) : 0.f;
            } else {
              const uint4 mk =
                  *reinterpret_cast<const uint4 *>(A.mask + ((size_t)(c0 / 8) * npix + p) * 8);
              const unsigned mw[4] = {mk.x, mk.y, mk.z, mk.w};
#pragma unroll
              for (int j = 0; j < 8; ++j) {
                const unsigned short bits = (unsigned short)(mw[j >> 1] >> (16 * (j & 1)));
                const bool pos = __bfloat162float(__ushort_as_bfloat16(bits)) > 0.f;
                v[j] = (c0 + j < A.nout && pos) ? accv[c0 + j] : 0.f;
              }
            }
            *reinterpret_cast<uint4 *>(A.out16 + ((size_t)(c0 / 8) * npix + p) * 8) =
                make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]),
                           pack_bf16(v[6], v[7]));
          }
        }
      }
    }
  }
  umma_fence_before();
  __syncthreads();
  umma_fence_after();
  if (warp == kMmaWarp) umma_dealloc(tmem, 64);
}

// ---------------------------------------------------------------------------
// Weight and bias gradient of one layer on the tensor cores.
//   D[m][co] = sum_p A[m][p] * dz[p][co],  m = tap * Csi + ci  (A[m][p] =
//   a[p + off(tap)][ci]),  m = taps Csi: a row of ones (bias gradient).
// Both operands MN-major: each 8-channel slice copied by TMA is one MN
// group of 8 rows x 128 pixels (core matrices 128 bytes apart along K, MN
// groups one 2048-byte slice apart).  One ring stage serves one M = 128
// slice of the rows for one tile: its 16 row groups (activation slices,
// the ones slice copied from a constant array, stale data for rows past
// the end, never stored) and the tile's Cout / 8 gradient slices.  Each
// CTA accumulates its tiles in tensor memory (one accumulator per M
// slice) and writes one partial sum.
// ---------------------------------------------------------------------------
struct WgradArgs {
  int Csi, Cin, Cso, Cout;
  int nz, nx, ny, taps, ntiles, tiles_z, tiles_x;
  int nmma;                      // M = 128 slices: ceil((taps Csi + 8) / 128)
  int ring;                      // shared-memory stages (<= kMaxRing)
  float *part;                   // [cta][10][kMaxC][kMaxC]
  int *err;
};
constexpr int kWgradStage = 20 * kChunk;   // 16 row groups + up to 4 gradient groups

size_t wgrad_smem_bytes(int ring) { return 1024 + (size_t)ring * kWgradStage; }

template <int NPO>
__global__ void __launch_bounds__(kWsThreads, 1)
    k_wgrad_umma(const __grid_constant__ CUtensorMap amap, const __grid_constant__ CUtensorMap dmap,
                 const __grid_constant__ CUtensorMap onemap, const WgradArgs A) {
  extern __shared__ unsigned char cnn_smem[];
  __shared__ __align__(8) unsigned long long full[kMaxRing], empty[kMaxRing], done;
  __shared__ unsigned tmem_base;
  __shared__ volatile int abort_flag;
  __shared__ volatile int mma_stages;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int G = A.taps * A.Csi / 8;               // activation groups; group G = ones
  unsigned char *ring = align1024(cnn_smem);
  if (tid == 0) {
    for (int q = 0; q < A.ring; ++q) {
      cnn_bar_init(&full[q], 1);
      cnn_bar_init(&empty[q], 1);
    }
    cnn_bar_init(&done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
    mma_stages = 0;
  }
  if (warp == kMmaWarp) umma_alloc(&tmem_base, 256);
  umma_fence_before();
  __syncthreads();
  umma_fence_after();
  const unsigned tmem = tmem_base;
  const int first = blockIdx.x, stride = gridDim.x;
  const int nmine = first < A.ntiles ? (A.ntiles - 1 - first) / stride + 1 : 0;
  if (warp == kProducerWarp) {
    if (lane == 0) {
      const int ng = A.Csi / 8;
      int q = 0;
      bool ok = true;
      for (int i = 0; i < nmine && ok; ++i) {
        const int t = first + i * stride;
        const int z0 = (t % A.tiles_z) * kTZ, x0 = ((t / A.tiles_z) % A.tiles_x) * kTX;
        const int y0 = t / (A.tiles_z * A.tiles_x);
        for (int j = 0; j < A.nmma; ++j, ++q) {
          const int slot = q % A.ring;
          if (q >= A.ring && !(ok = cnn_wait(&empty[slot], ((q / A.ring) - 1) & 1, &abort_flag)))
            break;
          unsigned char *dst = ring + (size_t)slot * kWgradStage;
          const int g1 = min(16 * j + 16, G + 1);
          cnn_expect_tx(&full[slot], (unsigned)((g1 - 16 * j + A.Cso / 8) * kChunk));
          // One tensor copy per tap (its ng channel-group slices; 16 is a
          // multiple of ng), the ones slice, then the gradient's slices.
          for (int g = 16 * j; g < g1; g += (g < G ? ng : 1)) {
            unsigned char *gd = dst + (size_t)(g - 16 * j) * kChunk;
            if (g < G) {
              int dz, dx, dy;
              tap_off(g / ng, A.taps, dz, dx, dy);
              cnn_tma4(gd, &amap, 0, z0 + dz, x0 + dx, y0 + dy, &full[slot]);
            } else {
              cnn_tma4(gd, &onemap, 0, 0, 0, 0, &full[slot]);
            }
          }
          cnn_tma4(dst + (size_t)16 * kChunk, &dmap, 0, z0, x0, y0, &full[slot]);
        }
      }
      if (!ok) {
        abort_flag = 1;
        atomicOr(A.err, 1);
      }
      if (abort_flag)
        for (int r = max(mma_stages, q - A.ring); r < q; ++r)
          umma_mbar_wait(&full[r % A.ring], (r / A.ring) & 1);
    }
  } else if (warp == kMmaWarp) {
    if (lane == 0) {
      constexpr uint32_t idesc = umma_idesc_bf16_mn(kTile, NPO);
      int q = 0;
      bool ok = true, any = false;
      for (int i = 0; i < nmine && ok; ++i)
        for (int j = 0; j < A.nmma; ++j, ++q) {
          const int slot = q % A.ring;
          if (!(ok = cnn_wait(&full[slot], (q / A.ring) & 1, &abort_flag))) break;
          mma_stages = q + 1;
          umma_fence_after();
          const unsigned sa = umma_su32(ring + (size_t)slot * kWgradStage);
          const unsigned sb = sa + 16 * kChunk;
          // MN-major, no swizzle: the leading byte offset is the step
          // between 8-row core-matrix groups along K (128 bytes here), the
          // stride byte offset the step between 8-element groups along M / N
          // (one 2048-byte slice).
#pragma unroll
          for (int ks = 0; ks < kTile / 16; ++ks)
            umma_bf16(tmem + j * NPO, umma_smem_desc(sa + ks * 256, 128, kChunk),
                      umma_smem_desc(sb + ks * 256, 128, kChunk), idesc, i > 0 || ks > 0);
          umma_commit(&empty[slot]);
          any = true;
        }
      if (!ok) {
        abort_flag = 1;
        atomicOr(A.err, 1);
      }
      if (any) umma_commit(&done);
      else cnn_arrive(&done);
    }
  } else if (nmine > 0) {
    // Epilogue: thread = accumulator lane = row (tap, ci) within a slice.
    bool ok = cnn_wait(&done, 0, &abort_flag) && !abort_flag;
    ok = __all_sync(0xffffffffu, ok);
    umma_fence_after();
    if (ok) {
      float *P = A.part + (size_t)blockIdx.x * kWgradSlots;
      for (int j = 0; j < A.nmma; ++j) {
        float accv[NPO];
        const unsigned ta = tmem + ((unsigned)(warp * 32) << 16) + j * NPO;
        umma_ld16(ta, accv);
        if (NPO == 32) umma_ld16(ta + 16, accv + 16);
        const int m = j * kTile + tid;
        if (m < A.taps * A.Csi) {
          const int tap = m / A.Csi, ci = m % A.Csi;
          if (ci < A.Cin)
#pragma unroll
            for (int co = 0; co < NPO; ++co)
              if (co < A.Cout) P[(size_t)tap * kMaxC * kMaxC + co * kMaxC + ci] = accv[co];
        } else if (m == A.taps * A.Csi) {
#pragma unroll
          for (int co = 0; co < NPO; ++co)
            if (co < A.Cout) P[(size_t)A.taps * kMaxC * kMaxC + co * kMaxC] = accv[co];
        }
      }
    } else if (lane == 0) {
      abort_flag = 1;
      atomicOr(A.err, 1);
    }
  }
  umma_fence_before();
  __syncthreads();
  umma_fence_after();
  if (warp == kMmaWarp) {
    // A give-up left products in flight: wait (bounded) for the last commit.
    if (abort_flag && lane == 0) umma_mbar_wait(&done, 0);
    __syncwarp();
    umma_dealloc(tmem, 256);
  }
}

// Sums the per-CTA partials in CTA order into the layer's gradient buffer
// (FP32, [co][tap][ci] then bias[co]) - added to what it holds.  Block
// `taps` is the bias.
__global__ void k_wgrad_sum(const float *__restrict__ part, int nchunk, int Cout, int Cin,
                            int taps, float *__restrict__ gw) {
  const int tap = blockIdx.x, t = threadIdx.x;
  const int co = t / kMaxC, ci = t % kMaxC;
  if (co >= Cout || (tap == taps ? ci != 0 : ci >= Cin)) return;
  float s = 0.f;
  for (int c = 0; c < nchunk; ++c) s += part[(size_t)c * kWgradSlots + tap * kMaxC * kMaxC + t];
  if (tap == taps) gw[(size_t)Cout * taps * Cin + co] += s;
  else gw[((size_t)co * taps + tap) * Cin + ci] += s;
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
// (out - target) / npix as BF16 in channel 0 of a 16-channel tensor (two
// planes, zero elsewhere), and per-block FP64 partial sums of
// (out - target)^2.
__global__ void k_loss(const float *__restrict__ out, const float *__restrict__ tgt, int npix,
                       __nv_bfloat16 *__restrict__ db, double *__restrict__ part) {
  __shared__ double red[256];
  double s = 0.0;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
    const float e = out[p] - tgt[p];
    s += (double)e * (double)e;
    *reinterpret_cast<uint4 *>(db + (size_t)p * 8) =
        make_uint4(pack_bf16(e / (float)npix, 0.f), 0u, 0u, 0u);
    *reinterpret_cast<uint4 *>(db + ((size_t)npix + p) * 8) = make_uint4(0u, 0u, 0u, 0u);
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
                               int taps, int NPo, int KPf, int NPi, int KPb,
                               __nv_bfloat16 *__restrict__ wf, __nv_bfloat16 *__restrict__ wb) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < NPo * KPf; q += gridDim.x * blockDim.x) {
    const int n = q / KPf, k = q % KPf;
    const int tap = k / Csi, ci = k % Csi;
    float v = 0.f;
    if (n < Cout && tap < taps && ci < Cin) v = w[((size_t)n * taps + tap) * Cin + ci];
    wf[umma_off(n, k, NPo) >> 1] = __float2bfloat16(v);
  }
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < NPi * KPb; q += gridDim.x * blockDim.x) {
    const int n = q / KPb, k = q % KPb;
    const int tap = k / Cso, co = k % Cso;
    float v = 0.f;
    if (n < Cin && tap < taps && co < Cout) v = w[((size_t)co * taps + tap) * Cin + n];
    wb[umma_off(n, k, NPi) >> 1] = __float2bfloat16(v);
  }
}

int nblk(long long n) { return (int)std::min<long long>(4096, (n + 255) / 256); }

// BF16 tensor map over Cs / 8 channel-group planes: dimensions (8 nz: z
// and the 8 channels flattened, nx, ny, Cs / 8), box 8 kTZ x cols x 1 x
// planes (cols rows of 512 bytes per plane), zero fill outside.
bool encode_act_map(CUtensorMap *m, const __nv_bfloat16 *base, int Cs, int nz, int nx, int ny,
                    int planes, int cols = kTX) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[4] = {(cuuint64_t)nz * 8, (cuuint64_t)nx, (cuuint64_t)ny,
                              (cuuint64_t)Cs / 8};
  const cuuint64_t strides[3] = {(cuuint64_t)nz * 16, (cuuint64_t)nz * nx * 16,
                                 (cuuint64_t)nz * nx * ny * 16};
  const cuuint32_t box[4] = {8 * kTZ, (cuuint32_t)cols, 1, (cuuint32_t)planes};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<__nv_bfloat16 *>(base), dims,
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
  kernel<<<grid, kWsThreads, smem, s>>>(m0, a);
  return cudaGetLastError();
}

// One convolution: input tensor (Cs channels) -> MODE's outputs.
cudaError_t launch_conv(int dev, int mode, int NP, const __nv_bfloat16 *in, int Cs, int nz, int nx,
                        int ny, int taps, ConvArgs a, cudaStream_t s) {
  CUtensorMap m;
  if (!encode_act_map(&m, in, Cs, nz, nx, ny, Cs / 8, kConvCols)) return cudaErrorInvalidValue;
  a.Cs = Cs;
  a.nz = nz;
  a.nx = nx;
  a.ny = ny;
  a.taps = taps;
  a.kp = r16(taps * Cs);
  a.tiles_z = (nz + kTZ - 1) / kTZ;
  a.tiles_x = (nx + kTX - 1) / kTX;
  a.ntiles = a.tiles_z * a.tiles_x * ny;
  // A ring of about 110 KB per CTA (two CTAs per SM); stages of one tap.
  const size_t stage = (size_t)(Cs / 8) * kConvPlane;
  a.ring = (int)std::max<size_t>(
      2, std::min<size_t>(kMaxRing, (110u * 1024u - 1024u - conv_wbytes(NP, a.kp)) / stage));
  const size_t smem = conv_smem_bytes(NP, a.kp, Cs, a.ring);
  const int per_sm = std::max<int>(1, std::min<int>(2, (int)((227u * 1024u) / smem)));
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
                         int Cout, int nz, int nx, int ny, int taps,
                         const __nv_bfloat16 *ones, float *part, int *err, cudaStream_t s,
                         int *nchunk) {
  WgradArgs w;
  w.Csi = cstore(Cin);
  w.Cin = Cin;
  w.Cso = cstore(Cout);
  w.Cout = Cout;
  w.nz = nz;
  w.nx = nx;
  w.ny = ny;
  w.taps = taps;
  w.tiles_z = (nz + kTZ - 1) / kTZ;
  w.tiles_x = (nx + kTX - 1) / kTX;
  w.ntiles = w.tiles_z * w.tiles_x * ny;
  w.nmma = (taps * w.Csi + 8 + kTile - 1) / kTile;
  w.ring = 5;
  w.part = part;
  w.err = err;
  CUtensorMap ma, md, mo;
  if (!encode_act_map(&ma, a, w.Csi, nz, nx, ny, w.Csi / 8) ||
      !encode_act_map(&md, dz, w.Cso, nz, nx, ny, w.Cso / 8) ||
      !encode_act_map(&mo, ones, 8, kTZ, kTX, 1, 1))
    return cudaErrorInvalidValue;
  const int NPO = r16(Cout);
  const size_t smem = wgrad_smem_bytes(w.ring);
  const int grid = std::min(w.ntiles, num_sms(dev));
  *nchunk = grid;
  cudaError_t e;
  if (NPO == 16) {
    e = cudaFuncSetAttribute(k_wgrad_umma<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return e;
    k_wgrad_umma<16><<<grid, kWsThreads, smem, s>>>(ma, md, mo, w);
  } else {
    e = cudaFuncSetAttribute(k_wgrad_umma<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return e;
    k_wgrad_umma<32><<<grid, kWsThreads, smem, s>>>(ma, md, mo, w);
  }
  return cudaGetLastError();
}

}  // namespace

struct sw_cnn {
  sw_ctx *ctx = nullptr;
  int nl = 0;
  int taps = 9;                        // 9: 3 x 3 kernels on images, 27: 3 x 3 x 3 on volumes
  std::vector<int> ch;                 // nl + 1 channel counts
  std::vector<size_t> woff;            // offset of layer l in the packed weights
  size_t nw = 0;                       // packed FP32 weights (w then b per layer)
  float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
  std::vector<__nv_bfloat16 *> wf, wb; // BF16 GEMM copies per layer
  int step = 0;
  // Per-image buffers (grow-only).
  size_t cap = 0;
  std::vector<__nv_bfloat16 *> a;      // layer inputs, cstore(ch[l]) / 8 channel-group planes
  __nv_bfloat16 *dz[2] = {nullptr, nullptr};   // gradients, up to cstore(max ch) / 8 planes
  float *out32 = nullptr, *in32 = nullptr, *tgt = nullptr, *part = nullptr;
  double *lpart = nullptr;
  int *err = nullptr;
  __nv_bfloat16 *ones = nullptr;       // one 8-channel tile of BF16 ones (bias gradient)
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
  for (int c : n->ch) cmax = std::max(cmax, cstore(c));
  n->a.assign(n->nl, nullptr);
  for (int l = 0; l < n->nl && ok; ++l)
    ok = ck(cudaMalloc(&n->a[l], npix * cstore(n->ch[l]) * sizeof(__nv_bfloat16)));
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
    const int T = n->taps;
    k_weights_bf16<<<16, 256, 0, s>>>(n->w + n->woff[l], Cout, Cin, cstore(Cin), cstore(Cout), T,
                                      r16(Cout), r16(T * cstore(Cin)), r16(Cin), r16(T * cstore(Cout)),
                                      n->wf[l], n->wb[l]);
    n->ctx->stats.launches_total++;
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SW_OK : cnn_fail(n, e, "cnn weights");
}

// Forward pass of one image (volume) already packed into n->a[0]; output
// in n->out32.
int forward(sw_cnn *n, int nz, int nx, int ny) {
  cudaStream_t s = n->ctx->stream;
  const int dev = n->ctx->device;
  const int T = n->taps;
  cudaError_t e;
  for (int l = 0; l < n->nl; ++l) {
    const int Cin = n->ch[l], Cout = n->ch[l + 1];
    const bool last = l + 1 == n->nl;
    ConvArgs a{};
    a.mirror = 0;
    a.W = n->wf[l];
    a.bias = n->w + n->woff[l] + (size_t)Cout * T * Cin;
    a.nout = Cout;
    a.cs_out = cstore(Cout);
    a.out32 = last ? n->out32 : nullptr;
    a.out16 = last ? nullptr : n->a[l + 1];
    a.err = n->err;
    const uint64_t np = (uint64_t)nz * nx * ny;
    const uint64_t bytes = np * cstore(Cin) * 2 + (last ? np * Cout * 4 : np * cstore(Cout) * 2);
    if ((e = timed_launch(n, bytes, 2 * np * Cout * T * Cin, [&] {
           return launch_conv(dev, last ? kFwdLast : kFwdHidden, r16(Cout), n->a[l], cstore(Cin), nz,
                              nx, ny, T, a, s);
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
int gradient(sw_cnn *n, int nbatch, int nz, int nx, int ny, const float *in, const float *target,
             double *loss) {
  cudaStream_t s = n->ctx->stream;
  const int dev = n->ctx->device;
  const int T = n->taps;
  const size_t npix = (size_t)nz * nx * ny;
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
    k_pack_input<<<nblk((long long)npix * cstore(n->ch[0])), 256, 0, s>>>(
        n->in32, n->ch[0], cstore(n->ch[0]), (int)npix, n->a[0]);
    n->ctx->stats.launches_total++;
    if ((st = forward(n, nz, nx, ny))) return st;
    // d loss / d output (one channel), FP64 loss partials.
    int cur = 0;
    k_loss<<<lblocks, 256, 0, s>>>(n->out32, n->tgt, (int)npix, n->dz[cur], n->lpart);
    n->ctx->stats.launches_total++;
    for (int l = n->nl - 1; l >= 0; --l) {
      const int Cin = n->ch[l], Cout = n->ch[l + 1];
      int nchunk = 0;
      const uint64_t np = (uint64_t)npix;
      if ((e = timed_launch(n, np * (cstore(Cin) + cstore(Cout)) * 2, 2 * np * T * Cin * Cout, [&] {
             return launch_wgrad(dev, n->a[l], Cin, n->dz[cur], Cout, nz, nx, ny, T, n->ones,
                                 n->part, n->err, s, &nchunk);
           })) != cudaSuccess)
        return cnn_fail(n, e, "cnn wgrad");
      k_wgrad_sum<<<T + 1, kMaxC * kMaxC, 0, s>>>(n->part, nchunk, Cout, Cin, T,
                                                  n->g + n->woff[l]);
      n->ctx->stats.launches_total++;
      if (l == 0) break;
      // Input gradient: mirrored taps, transposed weights, then ReLU' of
      // the layer input, into the other gradient buffer.
      ConvArgs a{};
      a.mirror = 1;
      a.W = n->wb[l];
      a.bias = nullptr;
      a.nout = Cin;
      a.cs_out = cstore(Cin);
      a.out16 = n->dz[cur ^ 1];
      a.mask = n->a[l];
      a.err = n->err;
      if ((e = timed_launch(n, np * (cstore(Cout) + 2 * cstore(Cin)) * 2, 2 * np * Cin * T * Cout, [&] {
             return launch_conv(dev, kBwd, r16(Cin), n->dz[cur], cstore(Cout), nz, nx, ny, T, a, s);
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

int create_net(sw_ctx *c, int nlayers, const int *channels, uint64_t seed, int taps,
               sw_cnn **out) {
  if (!c || !channels || !out || nlayers < 1 || nlayers > 16) return SW_BAD_PARAM;
  *out = nullptr;
  for (int l = 0; l <= nlayers; ++l)
    if (channels[l] < 1 || channels[l] > kMaxC)
      return fail(c, SW_BAD_PARAM, "cnn channels must be 1..32");
  cudaSetDevice(c->device);
  sw_cnn *n = new sw_cnn();
  n->ctx = c;
  n->nl = nlayers;
  n->taps = taps;
  n->ch.assign(channels, channels + nlayers + 1);
  for (int l = 0; l < nlayers; ++l) {
    n->woff.push_back(n->nw);
    n->nw += (size_t)n->ch[l + 1] * taps * n->ch[l] + n->ch[l + 1];
  }
  // He initialisation, zero biases.
  std::vector<float> h(n->nw, 0.f);
  std::mt19937_64 rng(seed);
  for (int l = 0; l < nlayers; ++l) {
    const int Cin = n->ch[l], Cout = n->ch[l + 1];
    std::normal_distribution<float> nd(0.f, std::sqrt(2.f / ((float)taps * Cin)));
    for (int q = 0; q < Cout * taps * Cin; ++q) h[n->woff[l] + q] = nd(rng);
  }
  auto ck = [](cudaError_t e) { return e == cudaSuccess; };
  bool ok = ck(cudaMalloc(&n->w, n->nw * 4)) && ck(cudaMalloc(&n->g, n->nw * 4)) &&
            ck(cudaMalloc(&n->m, n->nw * 4)) && ck(cudaMalloc(&n->v, n->nw * 4)) &&
            ck(cudaMalloc(&n->err, sizeof(int)));
  n->wf.assign(nlayers, nullptr);
  n->wb.assign(nlayers, nullptr);
  for (int l = 0; l < nlayers && ok; ++l) {
    const int Cin = n->ch[l], Cout = n->ch[l + 1];
    ok = ck(cudaMalloc(&n->wf[l], (size_t)r16(Cout) * r16(taps * cstore(Cin)) * 2)) &&
         ck(cudaMalloc(&n->wb[l], (size_t)r16(Cin) * r16(taps * cstore(Cout)) * 2));
  }
  const std::vector<unsigned short> one(8 * kTile, (unsigned short)0x3f80);   // BF16 1.0
  ok = ok && ck(cudaMalloc(&n->ones, one.size() * 2)) &&
       ck(cudaMemcpy(n->ones, one.data(), one.size() * 2, cudaMemcpyHostToDevice));
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

// Shared body of the image (ny = 1, 3 x 3 network) and volume (3 x 3 x 3
// network) entry points.
int cnn_forward(sw_cnn *n, int nz, int nx, int ny, const float *in, float *out) {
  if (n->ch[n->nl] != 1) return fail(n->ctx, SW_BAD_PARAM, "cnn output must have one channel");
  cudaSetDevice(n->ctx->device);
  cudaStream_t s = n->ctx->stream;
  const size_t npix = (size_t)nz * nx * ny;
  int st = ensure_images(n, npix);
  if (st) return st;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(n->in32, in, npix * n->ch[0] * 4, cudaMemcpyHostToDevice, s)) !=
      cudaSuccess)
    return cnn_fail(n, e, "cnn input");
  k_pack_input<<<nblk((long long)npix * cstore(n->ch[0])), 256, 0, s>>>(n->in32, n->ch[0],
                                                                     cstore(n->ch[0]), (int)npix,
                                                                     n->a[0]);
  n->ctx->stats.launches_total++;
  if ((st = forward(n, nz, nx, ny))) return st;
  if ((e = cudaMemcpyAsync(out, n->out32, npix * 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return cnn_fail(n, e, "cnn output");
  return check_err(n);
}

int cnn_gradient(sw_cnn *n, int nbatch, int nz, int nx, int ny, const float *in,
                 const float *target, float *grad, double *loss) {
  if (n->ch[n->nl] != 1) return fail(n->ctx, SW_BAD_PARAM, "cnn output must have one channel");
  cudaSetDevice(n->ctx->device);
  int st = gradient(n, nbatch, nz, nx, ny, in, target, loss);
  if (st) return st;
  if ((st = check_err(n))) return st;
  std::vector<float> h(n->nw);
  if (cudaMemcpy(h.data(), n->g, n->nw * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return SW_CUDA_ERR;
  for (size_t q = 0; q < n->nw; ++q) grad[q] = h[q] / (float)nbatch;
  return SW_OK;
}

int cnn_train_step(sw_cnn *n, int nbatch, int nz, int nx, int ny, const float *in,
                   const float *target, float lr, double *loss) {
  if (n->ch[n->nl] != 1) return fail(n->ctx, SW_BAD_PARAM, "cnn output must have one channel");
  cudaSetDevice(n->ctx->device);
  cudaStream_t s = n->ctx->stream;
  int st = gradient(n, nbatch, nz, nx, ny, in, target, loss);
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

}  // namespace

extern "C" {

int sw_cnn_create(sw_ctx *c, int nlayers, const int *channels, uint64_t seed, sw_cnn **out) {
  return create_net(c, nlayers, channels, seed, 9, out);
}

int sw_cnn_create3d(sw_ctx *c, int nlayers, const int *channels, uint64_t seed, sw_cnn **out) {
  return create_net(c, nlayers, channels, seed, 27, out);
}

int sw_cnn_destroy(sw_cnn *n) {
  if (!n) return SW_OK;
  cudaSetDevice(n->ctx->device);
  cudaStreamSynchronize(n->ctx->stream);
  free_images(n);
  cudaFree(n->w); cudaFree(n->g); cudaFree(n->m); cudaFree(n->v); cudaFree(n->err);
  cudaFree(n->ones);
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
  if (n->taps != 9) return fail(n->ctx, SW_BAD_PARAM, "a 3x3x3 network takes volumes");
  return cnn_forward(n, nz, nx, 1, in, out);
}

int sw_cnn_gradient(sw_cnn *n, int nbatch, int nz, int nx, const float *in, const float *target,
                    float *grad, double *loss) {
  if (!n || !in || !target || !grad || nbatch < 1 || nz < 1 || nx < 1) return SW_BAD_PARAM;
  if (n->taps != 9) return fail(n->ctx, SW_BAD_PARAM, "a 3x3x3 network takes volumes");
  return cnn_gradient(n, nbatch, nz, nx, 1, in, target, grad, loss);
}

int sw_cnn_train_step(sw_cnn *n, int nbatch, int nz, int nx, const float *in,
                      const float *target, float lr, double *loss) {
  if (!n || !in || !target || nbatch < 1 || nz < 1 || nx < 1) return SW_BAD_PARAM;
  if (n->taps != 9) return fail(n->ctx, SW_BAD_PARAM, "a 3x3x3 network takes volumes");
  return cnn_train_step(n, nbatch, nz, nx, 1, in, target, lr, loss);
}

int sw_cnn_forward3d(sw_cnn *n, int nz, int nx, int ny, const float *in, float *out) {
  if (!n || !in || !out || nz < 1 || nx < 1 || ny < 1) return SW_BAD_PARAM;
  if (n->taps != 27) return fail(n->ctx, SW_BAD_PARAM, "a 3x3 network takes images");
  return cnn_forward(n, nz, nx, ny, in, out);
}

int sw_cnn_gradient3d(sw_cnn *n, int nbatch, int nz, int nx, int ny, const float *in,
                      const float *target, float *grad, double *loss) {
  if (!n || !in || !target || !grad || nbatch < 1 || nz < 1 || nx < 1 || ny < 1)
    return SW_BAD_PARAM;
  if (n->taps != 27) return fail(n->ctx, SW_BAD_PARAM, "a 3x3 network takes images");
  return cnn_gradient(n, nbatch, nz, nx, ny, in, target, grad, loss);
}

int sw_cnn_train_step3d(sw_cnn *n, int nbatch, int nz, int nx, int ny, const float *in,
                        const float *target, float lr, double *loss) {
  if (!n || !in || !target || nbatch < 1 || nz < 1 || nx < 1 || ny < 1) return SW_BAD_PARAM;
  if (n->taps != 27) return fail(n->ctx, SW_BAD_PARAM, "a 3x3 network takes images");
  return cnn_train_step(n, nbatch, nz, nx, ny, in, target, lr, loss);
}

}  // extern "C"
