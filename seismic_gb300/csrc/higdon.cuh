// higdon.cuh - the Higdon absorbing-boundary recurrence along one edge
// line (Boundary_3d, Boundary.f90:89-184,366-447) for the separate edge
// kernels (batch.cu).
#pragma once

#include <cstdint>

#include "batch.cuh"

namespace swave {

// One half line of the Higdon recurrence with all inputs loaded first:
// the 10 u2 and u1 values from 2 cells inside the innermost output to the
// outermost one, the two u3 values inside it and the 8 coefficients; then
// the 8 outputs in order in registers:
//   u3(i) = -(g1 u3(i+d) + g2 u3(i+2d) + g3 u2(i) + g4 u2(i+d) + g5 u2(i+2d)
//            + g6 u1(i) + g7 u1(i+d) + g8 u1(i+2d))
// summed left to right, d the step towards the interior.
__device__ __forceinline__ void higdon_half(const float *__restrict__ gc, long long cs,
                                            const float *__restrict__ u1,
                                            const float *__restrict__ u2, float *u3,
                                            long long pstart, long long dst) {
  float c[8], U2[10], U1[10];
#pragma unroll
  for (int q = 0; q < 8; ++q) c[q] = gc[q * cs];
#pragma unroll
  for (int m = 0; m < 10; ++m) {
    const long long pm = pstart - (long long)(m - 2) * dst;   // k = m - 2
    U2[m] = u2[pm];
    U1[m] = u1[pm];
  }
  float a = u3[pstart + dst], bq = u3[pstart + 2 * dst];
  float out[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    float r = c[0] * a;
    r = r + c[1] * bq;
    r = r + c[2] * U2[k + 2];
    r = r + c[3] * U2[k + 1];
    r = r + c[4] * U2[k];
    r = r + c[5] * U1[k + 2];
    r = r + c[6] * U1[k + 1];
    r = r + c[7] * U1[k];
    out[k] = -r;
    bq = a;
    a = out[k];
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) u3[pstart - (long long)k * dst] = out[k];
}

// One Higdon z half line (Boundary_3d, Boundary.f90:89-184) of column
// (j, k): the top (bottom = false) or bottom 8 cells of u3 from u2 and u1 of
// the column and the two u3 cells inside the edge.
__device__ __forceinline__ void higdon_zline(const ShotDev &S, int j, int k, bool bottom,
                                             const float *u1, const float *u2, float *u3) {
  const Geom &g = S.g;
  const int n2 = g.nmax2 - g.nmin2 + 1, n3 = g.nmax3 - g.nmin3 + 1;
  const long long cs = (long long)n2 * n3;
  const long long l = (long long)(j - g.nmin2) + (long long)n2 * (k - g.nmin3);
  if (bottom) {
    // Bottom half line: the last 10 cells of the padded column, in 8-byte
    // loads and stores when they start on an 8-byte boundary (n1p even).
    const long long pb = g.idx(g.nmax1 - 3, j, k) - 2;   // cell n1p - 10
    const float *gcb = S.gz + l + 8 * cs;
    if (((reinterpret_cast<uintptr_t>(u1 + pb) | reinterpret_cast<uintptr_t>(u2 + pb) |
          reinterpret_cast<uintptr_t>(u3 + pb)) & 7) != 0) {
      higdon_half(gcb, cs, u1, u2, u3, pb + 2, -1);
      return;
    }
    float c[8], col2[10], col1[10];
#pragma unroll
    for (int m = 0; m < 8; ++m) c[m] = gcb[m * cs];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const float2 a2 = reinterpret_cast<const float2 *>(u2 + pb)[v];
      const float2 a1 = reinterpret_cast<const float2 *>(u1 + pb)[v];
      col2[2 * v] = a2.x; col2[2 * v + 1] = a2.y;
      col1[2 * v] = a1.x; col1[2 * v + 1] = a1.y;
    }
    const float2 t3 = reinterpret_cast<const float2 *>(u3 + pb)[0];   // cells pb, pb + 1
    float a = t3.y, bq = t3.x, out[8];
    // U(m) = cell pb + m, as in higdon_half with dst = -1 and pstart = pb + 2.
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
      float r = c[0] * a;
      r = r + c[1] * bq;
      r = r + c[2] * col2[kk + 2];
      r = r + c[3] * col2[kk + 1];
      r = r + c[4] * col2[kk];
      r = r + c[5] * col1[kk + 2];
      r = r + c[6] * col1[kk + 1];
      r = r + c[7] * col1[kk];
      out[kk] = -r;
      bq = a;
      a = out[kk];
    }
    // out[kk] belongs at cell pb + 2 + kk.
#pragma unroll
    for (int v = 0; v < 4; ++v)
      reinterpret_cast<float2 *>(u3 + pb + 2)[v] = make_float2(out[2 * v], out[2 * v + 1]);
    return;
  }
  // Top half line: its cells are the first 12 of the padded column (the
  // column starts on a 128-byte boundary: ld1 is a multiple of 32), so the
  // inputs come in 16-byte loads and the 8 outputs go out in two 16-byte
  // stores; the arithmetic is higdon_half's.
  const long long cb = g.idx(g.lo1, j, k);   // pstart = cb + 7
  const float *gc = S.gz + l;
  if (((reinterpret_cast<uintptr_t>(u1 + cb) | reinterpret_cast<uintptr_t>(u2 + cb) |
        reinterpret_cast<uintptr_t>(u3 + cb)) & 15) != 0) {
    higdon_half(gc, cs, u1, u2, u3, cb + 7, 1);
    return;
  }
  float c[8], col2[12], col1[12];
#pragma unroll
  for (int m = 0; m < 8; ++m) c[m] = gc[m * cs];
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    const float4 a2 = reinterpret_cast<const float4 *>(u2 + cb)[v];
    const float4 a1 = reinterpret_cast<const float4 *>(u1 + cb)[v];
    col2[4 * v] = a2.x; col2[4 * v + 1] = a2.y; col2[4 * v + 2] = a2.z; col2[4 * v + 3] = a2.w;
    col1[4 * v] = a1.x; col1[4 * v + 1] = a1.y; col1[4 * v + 2] = a1.z; col1[4 * v + 3] = a1.w;
  }
  const float2 t3 = reinterpret_cast<const float2 *>(u3 + cb)[4];   // cells 8, 9
  float a = t3.x, bq = t3.y, out[8];
  // U(m) = column cell 9 - m (m = 0..9), as in higdon_half with dst = 1.
#pragma unroll
  for (int kk = 0; kk < 8; ++kk) {
    float r = c[0] * a;
    r = r + c[1] * bq;
    r = r + c[2] * col2[7 - kk];
    r = r + c[3] * col2[8 - kk];
    r = r + c[4] * col2[9 - kk];
    r = r + c[5] * col1[7 - kk];
    r = r + c[6] * col1[8 - kk];
    r = r + c[7] * col1[9 - kk];
    out[kk] = -r;
    bq = a;
    a = out[kk];
  }
  // out[kk] belongs at cell 7 - kk.
  reinterpret_cast<float4 *>(u3 + cb)[0] = make_float4(out[7], out[6], out[5], out[4]);
  reinterpret_cast<float4 *>(u3 + cb)[1] = make_float4(out[3], out[2], out[1], out[0]);
}

// One Higdon x half line of row i in plane k: the left (right = false) or
// right 8 cells.
__device__ __forceinline__ void higdon_xline(const ShotDev &S, int i, int k, bool right,
                                             const float *u1, const float *u2, float *u3) {
  const Geom &g = S.g;
  const int n1 = g.nmax1 - g.nmin1 + 1, n3 = g.nmax3 - g.nmin3 + 1;
  const long long cs = (long long)n1 * n3;
  const long long l = (long long)(i - g.nmin1) + (long long)n1 * (k - g.nmin3);
  const long long L = g.ld1;
  if (!right) higdon_half(S.gx + l, cs, u1, u2, u3, g.idx(i, g.nmin2 + 3, k), L);
  else higdon_half(S.gx + l + 8 * cs, cs, u1, u2, u3, g.idx(i, g.nmax2 - 3, k), -L);
}

}  // namespace swave
