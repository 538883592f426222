// tile2d2.cuh - two time steps per launch for 2D batches (temporal blocking).
//
// Each CTA (512 threads, one per SM) walks 64 x 64 output tiles of all shots
// of the batch.  A tile's pipeline stage holds, by tensor copies:
//   U2: u2 with an 8-cell halo, 80 x 80 floats;
//   V : the velocity with a 4-cell halo (forward stencil, 72 x 72) or an
//       8-cell halo (adjoint stencil, 80 x 80);
//   U1, U0: u1 and u0 with a 4-cell halo, 72 x 72 each.
// Step A (time step s) is computed over the tile grown by 4 cells on every
// side (72 x 72) into a shared buffer, with u_-1 read by each thread from
// global memory; tiles at the domain edges then run the Higdon recurrence
// of step A on that buffer.  Step B (step s + 1) is computed over the 64 x 64
// core from the buffer, so no step needs another CTA's results.  Both new
// levels are stored (step A's u3, step B's u4); the shots keep six
// time-level buffers, so the launch never overwrites one of its inputs.
// DRAM traffic per point and two steps: u2, u1, u0, u_-1 and the velocity
// read, two levels written = 28 B, against 48 B for two single-step launches;
// the 4-cell rings of step A are recomputed by the neighbouring tiles
// (72 x 72 of step A per 64 x 64 of output).  Each element's operations are
// those of the single-step kernel (tile2d.cuh), in the reference's order.
#pragma once

#include "tile2d.cuh"

namespace swave {

constexpr int TF_Z = 64, TF_X = 64;      // core tile
constexpr int TF_E = 72;                 // extended tile: core + 4 cells
constexpr int TF_H = 80;                 // u2 tile: core + 8 cells
constexpr int TF_EXT = TF_E * TF_E;      // 5184 floats
constexpr int TF_U2 = TF_H * TF_H;       // 6400 floats
constexpr int TF_THREADS = 512;
constexpr int TF_MAX_TILES_PER_CTA = 320;
constexpr int TF_A_GROUPS = TF_E / 4;                 // 18 row groups of step A
constexpr int TF_A_UNITS = TF_A_GROUPS * (TF_E / 2);  // x 36 column pairs = 648
constexpr int TF_A_ROUNDS = (TF_A_UNITS + TF_THREADS - 1) / TF_THREADS;

template <bool ADJ>
__host__ __device__ constexpr int tf_vel_floats() {
  return ADJ ? TF_U2 : TF_EXT;
}
// Stage layout: [U2 | V | U1 | U0].
template <bool ADJ>
__host__ __device__ constexpr int tf_stage_floats() {
  return TF_U2 + tf_vel_floats<ADJ>() + 2 * TF_EXT;
}
// Dynamic shared memory: two stages, the step-A buffer, the shot table, the
// per-step scalars of both steps, the tile list and two mbarriers.
template <bool ADJ>
__host__ __device__ constexpr size_t tf_smem_bytes() {
  return sizeof(float) * (2 * tf_stage_floats<ADJ>() + TF_EXT) + sizeof(T2Shot) * TF_MAX_SHOTS +
         sizeof(T2Step) * 2 * TF_MAX_SHOTS + sizeof(int) * (TF_MAX_TILES_PER_CTA + 8) + 64;
}

__device__ __forceinline__ int tf_z0(const T2Shot &h, int e) {
  return h.nmin1 - h.off1 + t2_tzi(e) * TF_Z;
}
__device__ __forceinline__ int tf_x0(const T2Shot &h, int e) {
  return h.nmin2 - h.off2 + t2_txi(e) * TF_X;
}
__device__ __forceinline__ bool tf_phys_tile(const T2Shot &h, int e) {
  const int z0 = tf_z0(h, e), x0 = tf_x0(h, e);
  return !(z0 + TF_Z - 1 < 1 || z0 > h.nz || x0 + TF_X - 1 < 1 || x0 > h.nx);
}

__device__ __forceinline__ void sts4(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }

// Tensor copies of one tile into a stage (one thread); the maps cover the
// shot's six time-level buffers.  The extended tile's
// first row and column relative to the padded array's origin (4 cells
// before the compute domain) are ze, xe; ze is a multiple of 4 (16 bytes).
template <bool ADJ>
__device__ __forceinline__ void tf_issue(const T2FMaps &M, const T2Shot &h, int s, int e,
                                         float *st, unsigned long long *bar) {
  constexpr unsigned bytes = 4u * (unsigned)tf_stage_floats<ADJ>();
  constexpr int nb = 6;
  const int ze = t2_tzi(e) * TF_Z - h.off1, xe = t2_txi(e) * TF_X - h.off2;
  mbar_expect_tx(bar, bytes);
  tma_2d(st, &M.m[2 * ((s + 3) % nb)], ze - 4, xe - 4, bar);
  float *v = st + TF_U2;
  if (ADJ) tma_2d(v, &M.m[13], ze - 4, xe - 4, bar);
  else tma_2d(v, &M.m[12], ze, xe, bar);
  float *u1 = v + tf_vel_floats<ADJ>();
  tma_2d(u1, &M.m[2 * ((s + 2) % nb) + 1], ze, xe, bar);
  tma_2d(u1 + TF_EXT, &M.m[2 * ((s + 1) % nb) + 1], ze, xe, bar);
}

// Laplacian part of rows i..i+3 of two adjacent columns (t2_pair_fast with
// the arrays' column strides as parameters): SU of the staged u, SV of the
// velocity read at every stencil point (adjoint), SC of the velocity read at
// the outputs (forward).  u2c receives the raw u of the two columns.
template <bool ADJ, int SU, int SV, int SC>
__device__ __forceinline__ void tf_pair(const T2Pairs &c, const float *col0, const float *vcol0,
                                        const float *vcore0, P2 sv[2][2], float4 u2c[2]) {
  float4 N[10];
#pragma unroll
  for (int m = 0; m < 10; ++m) N[m] = lds4(col0 + (m - 4) * SU);
  u2c[0] = N[4];
  u2c[1] = N[5];
  if (ADJ) {
    // w = (v*v)*u at every stencil point (FDderivatives.f90:847-891).
#pragma unroll
    for (int m = 0; m < 10; ++m) {
      const float4 v = lds4(vcol0 + (m - 4) * SV);
      const P2 a = s_mul(p_mul(lo2(v), lo2(v)), lo2(N[m]));
      const P2 b = s_mul(p_mul(hi2(v), hi2(v)), hi2(N[m]));
      N[m] = make_float4(a.x, a.y, b.x, b.y);
    }
  }
#pragma unroll
  for (int cc = 0; cc < 2; ++cc) {
    const float *col = col0 + cc * SU;
    float4 za = lds4(col - 4), zc = lds4(col + 4);
    if (ADJ) {
      const float *vcol = vcol0 + cc * SV;
      const float4 va = lds4(vcol - 4), vc = lds4(vcol + 4);
      const P2 a0 = s_mul(p_mul(lo2(va), lo2(va)), lo2(za));
      const P2 a1 = s_mul(p_mul(hi2(va), hi2(va)), hi2(za));
      const P2 c0 = s_mul(p_mul(lo2(vc), lo2(vc)), lo2(zc));
      const P2 c1 = s_mul(p_mul(hi2(vc), hi2(vc)), hi2(zc));
      za = make_float4(a0.x, a0.y, a1.x, a1.y);
      zc = make_float4(c0.x, c0.y, c1.x, c1.y);
    }
    const float4 zb = N[4 + cc];
    const P2 P[6] = {lo2(za), hi2(za), lo2(zb), hi2(zb), lo2(zc), hi2(zc)};
    P2 Q[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) Q[k] = p2(P[k].y, P[k + 1].x);
    P2 tzz[2], txx[2];
#pragma unroll
    for (int p = 0; p < 2; ++p) {
      P2 a = s_mul(c.cz[0], P[2 + p]);
      a = p_add(a, s_mul(c.cz[1], p_add(Q[2 + p], Q[1 + p])));
      a = p_add(a, s_mul(c.cz[2], p_add(P[3 + p], P[1 + p])));
      a = p_add(a, s_mul(c.cz[3], p_add(Q[3 + p], Q[p])));
      a = p_add(a, s_mul(c.cz[4], p_add(P[4 + p], P[p])));
      tzz[p] = a;
      txx[p] = s_mul(c.cx[0], P[2 + p]);
    }
#pragma unroll
    for (int l = 1; l <= 4; ++l) {
      const float4 rp = N[4 + cc + l], rm = N[4 + cc - l];
      txx[0] = p_add(txx[0], s_mul(c.cx[l], p_add(lo2(rp), lo2(rm))));
      txx[1] = p_add(txx[1], s_mul(c.cx[l], p_add(hi2(rp), hi2(rm))));
    }
    if (ADJ) {
      sv[cc][0] = p_add(txx[0], tzz[0]);
      sv[cc][1] = p_add(txx[1], tzz[1]);
    } else {
      const float4 vv = lds4(vcore0 + cc * SC);
      sv[cc][0] = p_mul(p_mul(lo2(vv), lo2(vv)), p_add(txx[0], tzz[0]));
      sv[cc][1] = p_mul(p_mul(hi2(vv), hi2(vv)), p_add(txx[1], tzz[1]));
    }
  }
}

// Injection of time sample it (Injection.f90:151-456,561-591) into rows
// i0..i0+3 of columns j0, j0+1: every cell adds its entries' terms in entry
// order, from the block `sub` of the precomputed terms or formed here.
__device__ __forceinline__ void tf_inject(const ShotDev &S, const T2Shot &h, int it, int sub,
                                          int i0, int j0, P2 sv[2][2]) {
  if (i0 + 3 < h.bi0 || i0 > h.bi1) return;
  int beg[2][4], end[2][4];
#pragma unroll
  for (int hh = 0; hh < 2; ++hh) {
    const int j = j0 + hh;
    const bool cin = j >= h.bj0 && j <= h.bj1 && j >= h.nmin2 && j <= h.nmax2;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = i0 + q;
      beg[hh][q] = end[hh][q] = 0;
      if (cin && i >= h.bi0 && i <= h.bi1) {
        const int bx = (i - h.bi0) + (h.bi1 - h.bi0 + 1) * (j - h.bj0);
        beg[hh][q] = S.inj_off[bx];
        end[hh][q] = S.inj_off[bx + 1];
      }
    }
  }
  const float *terms = S.inj_term + (long long)sub * S.inj_nterm;
  auto term = [&](int k) {
    if (!h.inj_direct) return terms[k];
    const InjEntry E = S.inj_ent[k];
    const float tr = S.src_tr[(long long)E.tr * S.nt + (it - 1)];
    return (((E.v2r * tr) * E.wz) * E.wx) * E.wy;
  };
#pragma unroll
  for (int hh = 0; hh < 2; ++hh) {
    float r[4] = {sv[hh][0].x, sv[hh][0].y, sv[hh][1].x, sv[hh][1].y};
#pragma unroll
    for (int q = 0; q < 4; ++q)
      for (int k = beg[hh][q]; k < end[hh][q]; ++k) r[q] = r[q] + term(k);
    sv[hh][0] = p2(r[0], r[1]);
    sv[hh][1] = p2(r[2], r[3]);
  }
}

// FD_2nd_time_derivative_grid (FDderivatives.f90:960-982) of one column of
// 4 rows: (20 u2 - 6 u1 - 4 u0 + u_-1 + k12 L) / 11.
__device__ __forceinline__ float4 tf_update(const T2Pairs &c, float4 u, float4 a1, float4 a0,
                                            float4 am, const P2 sv[2]) {
  P2 o[2];
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    P2 a = s_mul(20.0f, p ? hi2(u) : lo2(u));
    a = p_sub(a, s_mul(6.0f, p ? hi2(a1) : lo2(a1)));
    a = p_sub(a, s_mul(4.0f, p ? hi2(a0) : lo2(a0)));
    a = p_add(a, p ? hi2(am) : lo2(am));
    a = p_add(a, s_mul(c.k12, sv[p]));
    o[p] = p_mul(a, c.div11);
  }
  return make_float4(o[0].x, o[0].y, o[1].x, o[1].y);
}

// Snapshot, image and illumination values of a thread's elements for an
// imaging step (t2_img_load on a 64 x 64 tile: rows z0 + tz + 16m of
// columns x0 + tx + 32hh).
__device__ __forceinline__ void tf_img_load(const T2Shot &h, const T2Step &stp, int e, T2Img &P,
                                            int tid) {
  const int z0 = tf_z0(h, e), x0 = tf_x0(h, e);
  const int tz = tid & 15, tx = tid >> 4;
#pragma unroll
  for (int hh = 0; hh < 2; ++hh) {
    const int j = x0 + tx + 32 * hh;
    const long long pc = (long long)h.nz * (j - 1) - 1;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int i = z0 + tz + 16 * m;
      const bool ok = t2_col_ok(h, j) && t2_row_ok(h, i);
      P.w[hh][m] = ok ? stp.wimg[pc + i] : 0.f;
      P.im[hh][m] = ok ? stp.image[pc + i] : 0.f;
      P.il[hh][m] = ok ? stp.illum[pc + i] : 0.f;
    }
  }
}

// Snapshot saving (Extraction.f90:562-601) and RTM / LSRTM imaging
// (Imaging.f90:265 and 735) of a thread's elements (t2_snap_tile on a
// 64 x 64 tile); su points at the tile's first core cell of the step's u
// (column stride SU), sv at that of the velocity (stride SV).
template <int SU, int SV>
__device__ __forceinline__ void tf_snap(const T2Shot &h, const T2Step &stp, const T2Img &P, int e,
                                        const float *su, const float *svel, int tid) {
  const int z0 = tf_z0(h, e), x0 = tf_x0(h, e);
  const int tz = tid & 15, tx = tid >> 4;
#pragma unroll
  for (int hh = 0; hh < 2; ++hh) {
    const int jl = tx + 32 * hh, j = x0 + jl;
    if (!t2_col_ok(h, j)) continue;
    const long long pc = (long long)h.nz * (j - 1) - 1;
    const float taper = stp.taperx ? stp.taperx[j - 1] * stp.tapery0 : 1.f;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int r = tz + 16 * m, i = z0 + r;
      if (!t2_row_ok(h, i)) continue;
      const float u = su[jl * SU + r];
      if (stp.extract) stp.wsave[pc + i] = u;
      if (stp.img) {
        const float wsn = P.w[hh][m];
        float im = P.im[hh][m];
        if (stp.img == 1) {
          im = im + (u * wsn) * taper;
        } else {
          const float v = svel[jl * SV + r];
          im = im + (((2.0f * taper) * u) * wsn) / v;
        }
        stp.image[pc + i] = im;
        stp.illum[pc + i] = P.il[hh][m] + (wsn * wsn) * taper;
      }
    }
  }
}

// Higdon edges (Boundary_3d, Boundary.f90:89-184) of one level over the
// rows rlo..rhi and columns clo..chi of a tile at the domain edges: the z
// lines of its columns, a barrier, then the x lines of its rows (the
// reference's order).  U2(i, j) and U1(i, j) give the two previous levels,
// U3(i, j) reads and W3(i, j, v) writes the new one.  Called by all threads
// of the CTA (it contains a barrier).
template <class FU2, class FU1, class FU3, class FW3>
__device__ __forceinline__ void tf_edges(const T2Shot &h, bool top, bool bottom, bool left,
                                         bool right, int rlo, int rhi, int clo, int chi, FU2 U2,
                                         FU1 U1, FU3 U3, FW3 W3, int tid) {
  const int n1 = h.nmax1 - h.nmin1 + 1, n2 = h.nmax2 - h.nmin2 + 1;
  if (top || bottom) {
    // Threads 0..127: top z lines, 128..255: bottom z lines; one column each.
    const bool bot = tid >= 128;
    const int j = clo + (tid & 127);
    if (tid < 256 && (bot ? bottom : top) && j <= chi && j >= h.nmin2 && j <= h.nmax2) {
      const int dir = bot ? -1 : 1;                       // towards the interior
      const int p = bot ? h.nmax1 - 3 : h.nmin1 + 3;      // innermost output row
      float c[8], u2[10], u1[10], out[8];
      const float *gc = h.gz + (j - h.nmin2) + (bot ? 8 * n2 : 0);
#pragma unroll
      for (int q = 0; q < 8; ++q) c[q] = gc[q * n2];
#pragma unroll
      for (int m = 0; m < 10; ++m) {
        const int i = p - (m - 2) * dir;
        u2[m] = U2(i, j);
        u1[m] = U1(i, j);
      }
      t2_higdon8(c, u2, u1, U3(p + dir, j), U3(p + 2 * dir, j), out);
#pragma unroll
      for (int k = 0; k < 8; ++k) W3(p - k * dir, j, out[k]);
    }
  }
  __syncthreads();   // z lines done before the x lines read the corners
  if (left || right) {
    // Threads 0..127: left x lines, 128..255: right x lines; one row each.
    const bool rgt = tid >= 128;
    const int i = rlo + (tid & 127);
    if (tid < 256 && (rgt ? right : left) && i <= rhi && i >= h.nmin1 && i <= h.nmax1) {
      const int dir = rgt ? -1 : 1;
      const int p = rgt ? h.nmax2 - 3 : h.nmin2 + 3;      // innermost output column
      float c[8], u2[10], u1[10], out[8];
      const float *gc = h.gx + (i - h.nmin1) + (rgt ? 8 * n1 : 0);
#pragma unroll
      for (int q = 0; q < 8; ++q) c[q] = gc[q * n1];
#pragma unroll
      for (int m = 0; m < 10; ++m) {
        const int j = p - (m - 2) * dir;
        u2[m] = U2(i, j);
        u1[m] = U1(i, j);
      }
      t2_higdon8(c, u2, u1, U3(i, p + dir), U3(i, p + 2 * dir), out);
#pragma unroll
      for (int k = 0; k < 8; ++k) W3(i, p - k * dir, out[k]);
    }
  }
}

// The two steps of one tile from a completed stage.
template <bool ADJ>
__device__ __forceinline__ void tf_tile(const BatchTables &t, const T2Shot &h, const T2Step &sa,
                                        const T2Step &sb, int b, int s, int e, float *st, float *A,
                                        const float4 (&um1)[TF_A_ROUNDS][2], const T2Img &P,
                                        bool img_a, int tid) {
  const ShotDev &S = t.shots[b];
  const int z0 = tf_z0(h, e), x0 = tf_x0(h, e);
  const T2Pairs c = t2_pairs(h);
  const float *U2 = st;
  const float *V = st + TF_U2;
  const float *U1 = V + tf_vel_floats<ADJ>();   // U0 follows at U1 + TF_EXT
  const bool liveb = sb.live;
  const bool inj_a = h.inj_on && !(z0 + TF_Z + 3 < h.bi0 || z0 - 4 > h.bi1 ||
                                   x0 + TF_X + 3 < h.bj0 || x0 - 4 > h.bj1);
  const bool inj_b = h.inj_on && !(z0 + TF_Z - 1 < h.bi0 || z0 > h.bi1 ||
                                   x0 + TF_X - 1 < h.bj0 || x0 > h.bj1);
  // ---- step A over the extended tile (rows z0-4.., columns x0-4..) ----
#pragma unroll
  for (int rd = 0; rd < TF_A_ROUNDS; ++rd) {
    const int u = tid + rd * TF_THREADS;
    if (u >= TF_A_UNITS) break;
    const int rz = u % TF_A_GROUPS, cx = u / TF_A_GROUPS;
    const int i0 = z0 - 4 + 4 * rz, j0 = x0 - 4 + 2 * cx;
    float4 o[2] = {make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f)};
    if (i0 >= h.nmin1 && i0 <= h.nmax1) {
      P2 sv[2][2];
      float4 u2c[2];
      const float *col0 = U2 + (2 * cx + 4) * TF_H + 4 * rz + 4;
      if (ADJ) tf_pair<ADJ, TF_H, TF_H, TF_E>(c, col0, V + (2 * cx + 4) * TF_H + 4 * rz + 4,
                                              nullptr, sv, u2c);
      else tf_pair<ADJ, TF_H, TF_H, TF_E>(c, col0, nullptr, V + (2 * cx) * TF_E + 4 * rz, sv,
                                          u2c);
      if (inj_a) tf_inject(S, h, sa.it, 0, i0, j0, sv);
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const int j = j0 + hh;
        if (j < h.nmin2 || j > h.nmax2) continue;
        const float *cc = U1 + (2 * cx + hh) * TF_E + 4 * rz;
        float4 r = tf_update(c, u2c[hh], lds4(cc), lds4(cc + TF_EXT), um1[rd][hh], sv[hh]);
        // Rows beyond the compute domain are not stencil outputs.
        if (i0 + 1 > h.nmax1) r.y = 0.f;
        if (i0 + 2 > h.nmax1) r.z = 0.f;
        if (i0 + 3 > h.nmax1) r.w = 0.f;
        o[hh] = r;
      }
    }
    sts4(A + (2 * cx) * TF_E + 4 * rz, o[0]);
    sts4(A + (2 * cx + 1) * TF_E + 4 * rz, o[1]);
  }
  // Snapshot / imaging of step A from the staged u2.
  if ((sa.extract || sa.img) && tf_phys_tile(h, e)) {
    if (ADJ) tf_snap<TF_H, TF_H>(h, sa, P, e, U2 + 8 * TF_H + 8, V + 8 * TF_H + 8, tid);
    else tf_snap<TF_H, TF_E>(h, sa, P, e, U2 + 8 * TF_H + 8, V + 4 * TF_E + 4, tid);
  }
  __syncthreads();   // the step-A buffer is complete
  const int tzi = t2_tzi(e), txi = t2_txi(e);
  const bool top = tzi == 0, bottom = tzi == h.ntz - 1;
  const bool left = txi == 0, right = txi == h.ntx - 1;
  const bool edge = !h.rigid && (top || bottom || left || right);
  if (edge) {
    // Higdon of step A on the extended tile: u2 = U2 (origin z0-8, x0-8),
    // u1 = U1 (origin z0-4, x0-4), u3 = the step-A buffer.
    auto a2 = [&](int i, int j) { return U2[(j - x0 + 8) * TF_H + (i - z0 + 8)]; };
    auto a1 = [&](int i, int j) { return U1[(j - x0 + 4) * TF_E + (i - z0 + 4)]; };
    auto a3 = [&](int i, int j) { return A[(j - x0 + 4) * TF_E + (i - z0 + 4)]; };
    auto w3 = [&](int i, int j, float v) { A[(j - x0 + 4) * TF_E + (i - z0 + 4)] = v; };
    tf_edges(h, top, bottom, left, right, z0 - 4, z0 + TF_Z + 3, x0 - 4, x0 + TF_X + 3, a2, a1,
             a3, w3, tid);
    __syncthreads();
  }
  // ---- store step A's core, then step B over the core ----
  const long long L = h.ld1;
  // Six time-level buffers (ShotDev::nbuf = 6 for two-step runs).
  float *__restrict__ u3 = S.f[(s + 4) % 6];
  float *__restrict__ u4 = S.f[(s + 5) % 6];
  const int rz = tid & 15, cx = tid >> 4;
  const int i0 = z0 + 4 * rz, j0 = x0 + 2 * cx;
  const int row0 = i0 - (h.nmin1 - 4);   // padded row index, a multiple of 4
  {
    // Cells of the padded array: rows nmin1-4..nmax1+4, columns lo2..lo2+n2p-1.
    if (i0 >= h.nmin1 - 4 && i0 <= h.nmax1 + 4) {
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const int j = j0 + hh;
        if (j < h.lo2 || j >= h.lo2 + h.n2p) continue;
        const float4 v = lds4(A + (2 * cx + hh + 4) * TF_E + 4 * rz + 4);
        const long long off = row0 + L * (j - h.lo2);
        if (i0 + 3 <= h.nmax1 + 4) {
          *reinterpret_cast<float4 *>(u3 + off) = v;
        } else {
          const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (i0 + q <= h.nmax1 + 4) u3[off + q] = vv[q];
        }
      }
    }
  }
  if (!liveb) return;
  if (i0 >= h.nmin1 && i0 <= h.nmax1) {
    P2 sv[2][2];
    float4 u2c[2];
    const float *col0 = A + (2 * cx + 4) * TF_E + 4 * rz + 4;
    if (ADJ) tf_pair<ADJ, TF_E, TF_H, TF_E>(c, col0, V + (2 * cx + 8) * TF_H + 4 * rz + 8,
                                            nullptr, sv, u2c);
    else tf_pair<ADJ, TF_E, TF_H, TF_E>(c, col0, nullptr, V + (2 * cx + 4) * TF_E + 4 * rz + 4,
                                        sv, u2c);
    if (inj_b) tf_inject(S, h, sb.it, 1, i0, j0, sv);
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
      const int j = j0 + hh;
      if (j < h.nmin2 || j > h.nmax2) continue;
      const float4 a1 = lds4(U2 + (2 * cx + hh + 8) * TF_H + 4 * rz + 8);
      const float *cc = U1 + (2 * cx + hh + 4) * TF_E + 4 * rz + 4;
      const float4 r = tf_update(c, u2c[hh], a1, lds4(cc), lds4(cc + TF_EXT), sv[hh]);
      const long long off = row0 + L * (j - h.lo2);
      if (i0 + 3 <= h.nmax1) {
        *reinterpret_cast<float4 *>(u4 + off) = r;
      } else {
        const float rv[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (i0 + q <= h.nmax1) u4[off + q] = rv[q];
      }
    }
  }
  // Snapshot / imaging of step B from the step-A buffer.
  if ((sb.extract || sb.img) && tf_phys_tile(h, e)) {
    T2Img Q;
    if (sb.img && !img_a) Q = P;
    else if (sb.img) tf_img_load(h, sb, e, Q, tid);
    if (ADJ) tf_snap<TF_E, TF_H>(h, sb, Q, e, A + 4 * TF_E + 4, V + 8 * TF_H + 8, tid);
    else tf_snap<TF_E, TF_E>(h, sb, Q, e, A + 4 * TF_E + 4, V + 4 * TF_E + 4, tid);
  }
  if (edge) {
    // Higdon of step B: u2 = the step-A buffer, u1 = U2, u3 = the stored u4.
    __syncthreads();   // the tile's u4 values are stored
    auto b2 = [&](int i, int j) { return A[(j - x0 + 4) * TF_E + (i - z0 + 4)]; };
    auto b1 = [&](int i, int j) { return U2[(j - x0 + 8) * TF_H + (i - z0 + 8)]; };
    auto gidx = [&](int i, int j) {
      return (long long)(i - (h.nmin1 - 4)) + L * (long long)(j - h.lo2);
    };
    auto b3 = [&](int i, int j) { return u4[gidx(i, j)]; };
    auto w4 = [&](int i, int j, float v) { u4[gidx(i, j)] = v; };
    tf_edges(h, top, bottom, left, right, z0, z0 + TF_Z - 1, x0, x0 + TF_X - 1, b2, b1, b3, w4,
             tid);
  }
}

template <bool ADJ>
__device__ __forceinline__ void tile2d_fused(const BatchTables &t, int s_off, int n_tiles) {
  extern __shared__ __align__(128) float tf_smem[];
  constexpr int SF = tf_stage_floats<ADJ>();
  float *A = tf_smem + 2 * SF;
  T2Shot *shots = reinterpret_cast<T2Shot *>(A + TF_EXT);
  T2Step *steps = reinterpret_cast<T2Step *>(shots + TF_MAX_SHOTS);   // [2 b + sub]
  int *list = reinterpret_cast<int *>(steps + 2 * TF_MAX_SHOTS);
  int *nlist = list + TF_MAX_TILES_PER_CTA;
  int *abort_flag = nlist + 1;
  unsigned long long *full = reinterpret_cast<unsigned long long *>(
      reinterpret_cast<char *>(tf_smem) + tf_smem_bytes<ADJ>() - 64);
  const int tid = threadIdx.x;
  {
    const int *src = reinterpret_cast<const int *>(t.t2shots);
    int *dst = reinterpret_cast<int *>(shots);
    const int nw = t.nshots * (int)(sizeof(T2Shot) / sizeof(int));
    for (int q = tid; q < nw; q += TF_THREADS) dst[q] = src[q];
    for (int k = tid; blockIdx.x + k * gridDim.x < n_tiles && k < TF_MAX_TILES_PER_CTA;
         k += TF_THREADS)
      list[k] = t.tile_tab[blockIdx.x + k * gridDim.x];
    if (tid == 0) {
      mbar_init(&full[0], 1);
      mbar_init(&full[1], 1);
      mbar_fence_init();
      *abort_flag = 0;
    }
  }
  // Everything after this reads what the previous kernels of the step
  // sequence wrote (fields, injection terms, the step counter).
  pdl_wait();
  pdl_launch_dependents();
  const int s = *t.counter + s_off;
  __syncthreads();
  if (tid < 2 * t.nshots) steps[tid] = t2_step_of<ADJ>(t, shots[tid >> 1], tid >> 1, s + (tid & 1));
  __syncthreads();
  if (tid == 0) {
    // Tiles of shots whose first step is live with this stencil variant.
    int n = 0;
    for (int k = 0; blockIdx.x + k * gridDim.x < n_tiles && k < TF_MAX_TILES_PER_CTA; ++k) {
      const int e = list[k];
      if (steps[2 * t2_b(e)].live) list[n++] = e;
    }
    *nlist = n;
    if (n > 0)
      tf_issue<ADJ>(t.tfmaps[t2_b(list[0])], shots[t2_b(list[0])], s, list[0], tf_smem,
                    &full[0]);
  }
  __syncthreads();
  const int n = *nlist;
  for (int k = 0; k < n; ++k) {
    const int cur = k & 1;
    if (tid == 0 && k + 1 < n)
      tf_issue<ADJ>(t.tfmaps[t2_b(list[k + 1])], shots[t2_b(list[k + 1])], s, list[k + 1],
                    tf_smem + (cur ^ 1) * SF, &full[cur ^ 1]);
    const int e = list[k];
    const int b = t2_b(e);
    const T2Shot &h = shots[b];
    const T2Step &sa = steps[2 * b], &sb = steps[2 * b + 1];
    // u_-1 of step A and the imaging inputs, loaded before the stage is
    // waited for so that their latency overlaps the wait.
    float4 um1[TF_A_ROUNDS][2];
    {
      const float *__restrict__ f0 = t.shots[b].f[s % 6];
      const int z0 = tf_z0(h, e), x0 = tf_x0(h, e);
#pragma unroll
      for (int rd = 0; rd < TF_A_ROUNDS; ++rd) {
        const int u = tid + rd * TF_THREADS;
        const int rz = u % TF_A_GROUPS, cx = u / TF_A_GROUPS;
        const int i0 = z0 - 4 + 4 * rz, j0 = x0 - 4 + 2 * cx;
        const bool rows = u < TF_A_UNITS && i0 >= h.nmin1 && i0 <= h.nmax1;
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
          const int j = j0 + hh;
          um1[rd][hh] = make_float4(0.f, 0.f, 0.f, 0.f);
          if (rows && j >= h.nmin2 && j <= h.nmax2)
            um1[rd][hh] = *reinterpret_cast<const float4 *>(
                f0 + (i0 - (h.nmin1 - 4)) + (long long)h.ld1 * (j - h.lo2));
        }
      }
    }
    T2Img P;
    const bool img_a = sa.img != 0;
    if ((sa.img || sb.img) && tf_phys_tile(h, e)) tf_img_load(h, img_a ? sa : sb, e, P, tid);
    if (!mbar_wait(&full[cur], (unsigned)((k >> 1) & 1))) {
      atomicOr(t.err, 1);
      *abort_flag = 1;
    }
    tf_tile<ADJ>(t, h, sa, sb, b, s, e, tf_smem + cur * SF, A, um1, P, img_a, tid);
    __syncthreads();   // the stage and the step-A buffer are free for the next tiles
    if (*abort_flag) {
      if (tid == 0) {
        mbar_wait(&full[cur], (unsigned)((k >> 1) & 1));
        if (k + 1 < n) mbar_wait(&full[cur ^ 1], (unsigned)(((k + 1) >> 1) & 1));
      }
      break;
    }
  }
}

}  // namespace swave
