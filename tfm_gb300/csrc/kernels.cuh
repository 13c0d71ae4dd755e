// Device kernels of the GB300 Brownian-dynamics engine.
//
// One Heun step (ccp's stochastic Runge-Kutta, chrsim.cu:365-416) is
//   [scan -> scatter(r) -> pair -> update<1>] [scan -> scatter(er) -> pair -> update<2>]
// where
//   scan     turns per-cell bead counts (one byte per cell) into cell start
//            offsets (3 launches),
//   scatter  writes every bead into cell order (the sorted float4 copy),
//   pair     evaluates the excluded-volume / attraction forces over the
//            27-cell neighbourhood in cell order (chrsim.cu:224-317),
//   update   is the fused chain-order pass: bonded + bending (chrsim.cu:13-76),
//            wall (chrsim.cu:79-170), lamina binding (chrsim.cu:202-212,
//            261-273), counter-based noise (replaces chrsim.cu:336-361), the
//            integrator stage, and the cell count of the new position (the
//            histogram of the next counting sort, replacing sugrid.cu:15-77 and
//            the CUB radix sort of sugrid.cu:130).
// All kernels take a tile table: each CTA owns a contiguous bead range of one
// system, so per-system geometry is uniform across a CTA.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace ccpgpu {

enum : int {
  ERR_NAN = 0,       // non-finite position produced
  ERR_ESCAPE = 1,    // bead outside its cell grid (clamped to the border)
  ERR_SLOT = 2,      // scatter slot outside the system range (inconsistent counts)
  ERR_NOISE = 3,     // truncated normal needed more than NOISE_MAX_ATTEMPTS draws
  ERR_WALK = 4,      // a confined random walk used up its draw budget
  ERR_COUNT = 8,
};

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;                       // cells per thread
constexpr int SCAN_CHUNK = SCAN_THREADS * SCAN_ITEMS;  // cells per CTA
constexpr int SCAN_TOP_THREADS = 1024;

struct Tile {
  int32_t sys;    // system index
  int32_t begin;  // first bead (chain order) or slot (cell order) of the tile
};

// ------------------------------------------------------------------ helpers

__device__ __forceinline__ uint32_t wbits(float4 p) { return __float_as_uint(p.w); }

// Integer cell coordinate along one axis of a grid centred at the origin with
// cps cells per side (sugrid.cu:27-34 / chrsim.cu:292-293). Out-of-grid values
// are clamped to the border cell and reported.
__device__ __forceinline__ int cell_coord(float v, float inv_csl, int cps, bool &esc) {
  float c = floorf(__fmul_rn(v, inv_csl)) + (float)(cps >> 1);
  if (!(c >= 0.0f)) {
    esc = true;
    return 0;
  }
  if (c >= (float)cps) {
    esc = true;
    return cps - 1;
  }
  return (int)c;
}

struct CellXYZ {
  int x, y, z;
};

__device__ __forceinline__ CellXYZ cell_of(float4 p, const SysDesc &s, bool &esc) {
  CellXYZ c;
  c.x = cell_coord(p.x, s.inv_csl, s.cps, esc);
  c.y = cell_coord(p.y, s.inv_csl, s.cps, esc);
  c.z = cell_coord(p.z, s.inv_csl, s.cps, esc);
  return c;
}

__device__ __forceinline__ int cell_linear(CellXYZ c, const SysDesc &s) {
  return s.cell_off + (c.z * s.cps + c.y) * s.cps + c.x;
}

// Cell of a bead in the sort: the A beads (BF_HET) use the system's first
// grid, the other beads the second one when the layout is typed.
__device__ __forceinline__ int bead_cell(float4 p, const SysDesc &s, bool &esc) {
  int c = cell_linear(cell_of(p, s, esc), s);
  return (wbits(p) & BF_HET) ? c : c + s.cls_cells;
}

__device__ __forceinline__ void set_err(int *err, int code) {
  if (err[code] == 0) atomicExch(&err[code], 1);
}

// ---- well-conditioned FP32 building blocks
// Error of the rounded sum s = a + b (TwoSum, Knuth): a + b = s + err exactly.
__device__ __forceinline__ float two_sum_err(float a, float b, float s) {
  float t = __fsub_rn(s, a);
  return __fadd_rn(__fsub_rn(a, __fsub_rn(s, t)), __fsub_rn(b, t));
}

// a^2 + b^2 + c^2 - (kh + kl) from error-free products and sums: keeps full
// relative precision when the squared length is close to kh (bond lengths near
// l_0, beads near the wall), where the naive form cancels.
__device__ __forceinline__ float sq3_minus(float a, float b, float c, float kh, float kl) {
  float pa = __fmul_rn(a, a), ea = __fmaf_rn(a, a, -pa);
  float pb = __fmul_rn(b, b), eb = __fmaf_rn(b, b, -pb);
  float pc = __fmul_rn(c, c), ec = __fmaf_rn(c, c, -pc);
  float s1 = __fadd_rn(pa, pb), e1 = two_sum_err(pa, pb, s1);
  float s2 = __fadd_rn(s1, pc), e2 = two_sum_err(s1, pc, s2);
  float s3 = __fsub_rn(s2, kh), e3 = two_sum_err(s2, -kh, s3);
  float lo = __fadd_rn(__fadd_rn(__fadd_rn(ea, eb), __fadd_rn(ec, e1)),
                       __fsub_rn(__fadd_rn(e2, e3), kl));
  return __fadd_rn(s3, lo);
}

// R / d - 1 = (R^2 - d^2) / ((R + d) d) for the point (a, b, c) at distance d.
__device__ __forceinline__ float r_over_d_minus1(float R, float a, float b, float c, float d) {
  float rh = __fmul_rn(R, R), rl = __fmaf_rn(R, R, -rh);
  return -sq3_minus(a, b, c, rh, rl) / ((R + d) * d);
}

// Wang-Frenkel (rc = 2) coefficient e (18 d^4 - 96 d^2 + 96) / d^8 in the
// factored form 6 e (d^2 - 4)(3 d^2 - 4) / d^8 (roots at the cutoffs 2 and 2/sqrt(3)).
__device__ __forceinline__ float wf_coef(float e, float d2) {
  float i2 = 1.0f / d2, i4 = i2 * i2;
  return 6.0f * e * (__fsub_rn(d2, 4.0f) * __fmaf_rn(3.0f, d2, -4.0f)) * (i4 * i4);
}

// 2^(1/3), the squared distance of the Lennard-Jones force's zero (the WCA
// cutoff 2^(1/6)), as a pair of FP32 words, and its square.
constexpr float LJ_Z2_HI = 1.259921074e+00f;
constexpr float LJ_Z2_LO = -2.401870169e-08f;
constexpr float LJ_Z2_SQ = 1.587401032e+00f;

// d^2 - 2^(1/3) for the pair vector (dx, dy, dz), |components| < 2, without
// cancellation: each component is split as x = xh + xl with xh on a 2^-10
// grid (rounded by adding and subtracting 1.5 * 2^13), so xh^2 and the sum of
// the three are exact in FP32 and the sum minus 2^(1/3) is exact (Sterbenz)
// for d^2 within a factor 2 of it; x^2 - xh^2 = xl (xh + x) is small.
__device__ __forceinline__ float lj_zero_gap(float dx, float dy, float dz) {
  const float M = 12288.0f;
  float xh = __fsub_rn(__fadd_rn(dx, M), M), yh = __fsub_rn(__fadd_rn(dy, M), M),
        zh = __fsub_rn(__fadd_rn(dz, M), M);
  float sh = __fmaf_rn(zh, zh, __fmaf_rn(yh, yh, __fmul_rn(xh, xh)));
  float lo = __fmaf_rn(__fsub_rn(dx, xh), __fadd_rn(xh, dx),
                       __fmaf_rn(__fsub_rn(dy, yh), __fadd_rn(yh, dy),
                                 __fmaf_rn(__fsub_rn(dz, zh), __fadd_rn(zh, dz), -LJ_Z2_LO)));
  return __fadd_rn(__fsub_rn(sh, LJ_Z2_HI), lo);
}

// Lennard-Jones coefficient 24 e (2 / d^14 - 1 / d^8) = 24 e d^-8 (2 d^-6 - 1)
// for the pair vector (dx, dy, dz) with FP32 squared length d2. The factor
// 2 d^-6 - 1 cancels at the force's zero, the WCA cutoff of the repulsive
// class: from a rounded d2 it carries an absolute error of ~5e-7, up to
// 3e-6 kT/sigma on the pair force there. For that class (ZERO_GAP) it is
// formed as
//   2 d^-6 - 1 = -(d^2 - 2^(1/3)) (d^4 + 2^(1/3) d^2 + 2^(2/3)) d^-6
// from the error-free d^2 - 2^(1/3) above, so its error stays relative to
// itself. The attractive A-A class (half the well depth, cut at 2.5 sigma)
// keeps the plain form: its pairs near the zero are measured not to set the
// force error.
template <bool ZERO_GAP>
__device__ __forceinline__ float lj_coef(float e, float dx, float dy, float dz, float d2) {
  float i2 = 1.0f / d2, i6 = i2 * i2 * i2;
  float m;
  if (ZERO_GAP) {
    float q = __fmaf_rn(d2, __fadd_rn(d2, LJ_Z2_HI), LJ_Z2_SQ);
    m = -lj_zero_gap(dx, dy, dz) * q * i6;
  } else {
    m = __fmaf_rn(2.0f, i6, -1.0f);
  }
  return 24.0f * e * (i6 * i2) * m;
}

// Coefficient c of a pair force F_i = c (r_i - r_j) (chrsim.cu:174-198) for
// the pair vector (dx, dy, dz) of squared length d2.
template <int MODE>
__device__ __forceinline__ float pair_coef(float dx, float dy, float dz, float d2, bool hh,
                                           const ForceField &ff) {
  if (MODE == MODE_ICG) {
    // soft repulsion 128 (3 rco - 3 d) (chrsim.cu:189-198)
    if (d2 > ff.rc_icg * ff.rc_icg) return 0.0f;
    float d = sqrtf(d2);
    return ff.k_icg * (3.0f * ff.rc_icg - 3.0f * d);
  }
  float rc = hh ? ff.rc_att : ff.rc_rep;
  if (d2 > rc * rc) return 0.0f;
  if (ff.pot == POT_WF) return wf_coef(ff.e_att, d2);
  return hh ? lj_coef<false>(ff.e_att, dx, dy, dz, d2) : lj_coef<true>(ff.e_rep, dx, dy, dz, d2);
}

// Distance d of (a, b, c) from the origin and the gap g = R - d carried as a
// double-float gh + gl (pairs of FP32 words), from R^2 - d^2 formed without
// cancellation. The wall potentials depend on g^2 near their cutoffs, where a
// single-float g (rounding 6e-8) would leave ~1e-5 relative force error.
__device__ __forceinline__ void gap_df(float R, float a, float b, float c, float &dist,
                                       float &gh, float &gl) {
  float pa = __fmul_rn(a, a), ea = __fmaf_rn(a, a, -pa);
  float pb = __fmul_rn(b, b), eb = __fmaf_rn(b, b, -pb);
  float pc = __fmul_rn(c, c), ec = __fmaf_rn(c, c, -pc);
  float s1 = __fadd_rn(pa, pb), e1 = two_sum_err(pa, pb, s1);
  float s2 = __fadd_rn(s1, pc), e2 = two_sum_err(s1, pc, s2);
  float lo = __fadd_rn(__fadd_rn(ea, eb), __fadd_rn(ec, __fadd_rn(e1, e2)));
  float d2h = __fadd_rn(s2, lo), d2l = __fsub_rn(lo, __fsub_rn(d2h, s2));
  float dh = sqrtf(d2h);
  float dl = (dh > 0.0f) ? __fadd_rn(__fmaf_rn(-dh, dh, d2h), d2l) / (2.0f * dh) : 0.0f;
  float rh = __fmul_rn(R, R), rl = __fmaf_rn(R, R, -rh);
  float nh = __fsub_rn(rh, d2h);
  float nl = __fadd_rn(two_sum_err(rh, -d2h, nh), __fsub_rn(rl, d2l));
  float deh = __fadd_rn(R, dh);
  float del = __fadd_rn(two_sum_err(R, dh, deh), dl);
  float qh = nh / deh;
  float rr = __fsub_rn(__fadd_rn(__fmaf_rn(-qh, deh, nh), nl), __fmul_rn(qh, del));
  float ql = rr / deh;
  gh = __fadd_rn(qh, ql);
  gl = __fsub_rn(ql, __fsub_rn(gh, qh));
  dist = dh;
}

// Wall-particle vector v of ccp's nucleus + opening + bleb geometry
// (chrsim.cu:92-137; the ICG mode uses the bare sphere, chrsim.cu:148-163),
// with |v| = gh + gl. Returns false when v is not finite (no wall force,
// chrsim.cu:137).
template <int MODE>
__device__ __forceinline__ bool wall_vector(float3 r, const SysDesc &s, float3 &v, float &gh,
                                            float &gl) {
  float3 q = r;
  float R = s.R_n;
  bool sphere = true;
  if (MODE != MODE_ICG) {
    if (r.z < s.nod) {
      float d = sqrtf(r.x * r.x + r.y * r.y + r.z * r.z);
      if (!(r.z / d < s.noc)) {
        d = sqrtf(r.x * r.x + r.y * r.y);
        float k = -r_over_d_minus1(s.R_o, r.x, r.y, 0.0f, d);
        v = make_float3(r.x * k, r.y * k, r.z - s.nod);
        sphere = false;
      }
    } else {
      q = make_float3(r.x, r.y, r.z - (s.nod + s.bod));
      R = s.R_b;
      float d = sqrtf(q.x * q.x + q.y * q.y + q.z * q.z);
      if (!(-q.z / d < s.boc)) {
        d = sqrtf(q.x * q.x + q.y * q.y);
        float k = -r_over_d_minus1(s.R_o, q.x, q.y, 0.0f, d);
        v = make_float3(q.x * k, q.y * k, q.z + s.bod);
        sphere = false;
      }
    }
  }
  if (sphere) {
    float d;
    gap_df(R, q.x, q.y, q.z, d, gh, gl);
    float k = -gh / d;  // -(R/d - 1)
    v = make_float3(q.x * k, q.y * k, q.z * k);
    if (gh < 0.0f) {  // outside: |v| = d - R
      gh = -gh;
      gl = -gl;
    }
  } else {
    gh = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    gl = 0.0f;
  }
  float l = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
  return isfinite(l) && isfinite(gh);
}

// Wall force coefficient c (F = c v) from the double-float distance g = gh + gl
// (chrsim.cu:79-88 for the Wang-Frenkel form); the relaxation mode always uses
// ccp's soft Wang-Frenkel wall. Both forms are evaluated from g^2 without the
// cancellation at their cutoffs: WF 6e (g^2 - 4)(3 g^2 - 4) / g^8 and
// LJ 24e (2 - g^6) / g^14.
template <int MODE>
__device__ __forceinline__ float wall_coef(float gh, float gl, const ForceField &ff) {
  const bool wf = (MODE == MODE_ICG) || (ff.pot == POT_WF);
  const float e = (MODE == MODE_ICG) ? 1.0f : ff.e_w;
  if (gh > ((MODE == MODE_ICG) ? ICG_WALL_RC : ff.rc_w)) return 0.0f;
  float h2h = __fmul_rn(gh, gh);
  float h2l = __fadd_rn(__fmaf_rn(gh, gh, -h2h), 2.0f * gh * gl);
  float i2 = 1.0f / h2h, i4 = i2 * i2;
  if (wf) {
    float a = __fadd_rn(__fsub_rn(h2h, 4.0f), h2l);
    float b = __fadd_rn(__fmaf_rn(3.0f, h2h, -4.0f), 3.0f * h2l);
    return 6.0f * e * (a * b) * (i4 * i4);
  }
  float p1 = __fmul_rn(h2h, h2h), e1 = __fmaf_rn(h2h, h2h, -p1);
  float p2 = __fmul_rn(p1, h2h), e2 = __fmaf_rn(p1, h2h, -p2);
  float lo6 = __fadd_rn(__fadd_rn(e2, e1 * h2h), 3.0f * h2h * h2h * h2l);
  float m = __fsub_rn(__fsub_rn(2.0f, p2), lo6);
  float i6 = i4 * i2;
  return 24.0f * e * m * (i6 * i6 * i2);  // 1 / g^14
}

// Truncated standard normals for one bead and step: three Box-Muller normals
// from one Philox block, redrawn with the next attempt counter while any
// |z| > 5 (chrsim.cu:350-356 truncation on the component triple).
__device__ __forceinline__ float3 bead_noise(uint32_t bead, uint64_t step, uint32_t k0,
                                             uint32_t k1, int *err) {
  for (int a = 0; a < NOISE_MAX_ATTEMPTS; ++a) {
    U32x4 b = noise_bits(bead, (uint32_t)a, step, k0, k1);
    float r0 = sqrtf(-2.0f * logf(u01_open0(b.x)));
    float s0, c0;
    sincospif(2.0f * u01_open1(b.y), &s0, &c0);
    float r1 = sqrtf(-2.0f * logf(u01_open0(b.z)));
    float c1 = cospif(2.0f * u01_open1(b.w));
    float3 z = make_float3(r0 * c0, r0 * s0, r1 * c1);
    if (fabsf(z.x) <= NOISE_TRUNC && fabsf(z.y) <= NOISE_TRUNC && fabsf(z.z) <= NOISE_TRUNC)
      return z;
  }
  set_err(err, ERR_NOISE);
  return make_float3(0.0f, 0.0f, 0.0f);
}

// ------------------------------------------------------------------ count

// Cell histograms hold one byte per cell, four cells to a 32-bit word, so the
// scan reads one byte per cell. A cell of side ~ sigma holds a few beads; one
// that would pass 255 sets ERR_SLOT (the carry has spoiled its neighbour's
// count) and the run reports an inconsistent cell list. Returns the bead's
// rank in its cell.
__device__ __forceinline__ uint32_t cell_add(uint32_t *counts, int c, int *err) {
  const uint32_t sh = 8u * ((uint32_t)c & 3u);
  const uint32_t r = (atomicAdd(&counts[c >> 2], 1u << sh) >> sh) & 0xFFu;
  if (r == 0xFFu) set_err(err, ERR_SLOT);
  return r;
}

// Cell histogram of the current positions: rank[i] = position of bead i in
// its cell, counts[c] += 1. Used after positions are (re)loaded; during
// stepping the update kernel does this for the position it writes.
__global__ void k_count(const Tile *__restrict__ tiles, const SysDesc *__restrict__ sys,
                        const float4 *__restrict__ pos, uint32_t *__restrict__ counts,
                        uint32_t *__restrict__ rank, int *__restrict__ err) {
  Tile t = tiles[blockIdx.x];
  const SysDesc &s = sys[t.sys];
  int i = t.begin + threadIdx.x;
  if (i >= s.bead_off + s.n) return;
  bool esc = false;
  float4 p = pos[i];
  int c = bead_cell(p, s, esc);
  rank[i] = cell_add(counts, c, err);
  if (esc) set_err(err, ERR_ESCAPE);
}

// ------------------------------------------------------------------ scan

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
  int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t n = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += n;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix and writes the block total to *total.
template <int NT>
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *total) {
  __shared__ uint32_t wsum[NT / 32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t inc = warp_incl_scan(v);
  if (lane == 31) wsum[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    uint32_t w = (lane < NT / 32) ? wsum[lane] : 0u;
    uint32_t wi = warp_incl_scan(w);
    if (lane < NT / 32) wsum[lane] = wi - w;
    if (lane == NT / 32 - 1) *total = wi;
  }
  __syncthreads();
  uint32_t r = wsum[wid] + inc - v;
  __syncthreads();
  return r;
}

// Phase 1: per-CTA totals of SCAN_CHUNK cells (SCAN_ITEMS = 16 byte counts,
// one 16-byte load, per thread). counts is padded to a multiple of
// SCAN_CHUNK cells (zeros beyond n_cells).
__global__ void __launch_bounds__(SCAN_THREADS)
    k_scan_reduce(const uint32_t *__restrict__ counts, uint32_t *__restrict__ block_sums) {
  static_assert(SCAN_ITEMS == 16, "one uint4 of byte counts per thread");
  const uint4 q = reinterpret_cast<const uint4 *>(counts)[(size_t)blockIdx.x * SCAN_THREADS +
                                                         threadIdx.x];
  uint32_t v = __vsadu4(q.x, 0u) + __vsadu4(q.y, 0u) + __vsadu4(q.z, 0u) + __vsadu4(q.w, 0u);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __shared__ uint32_t ws[SCAN_THREADS / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < SCAN_THREADS / 32; ++w) t += ws[w];
    block_sums[blockIdx.x] = t;
  }
}

// Phase 2: one CTA scans the CTA totals in place (exclusive) and stores the
// grand total at block_sums[nb]. It also advances the step counter when the
// scan opens a new Heun step (bump != 0).
__global__ void __launch_bounds__(SCAN_TOP_THREADS)
    k_scan_top(uint32_t *__restrict__ block_sums, int nb, unsigned long long *step, int bump) {
  __shared__ uint32_t tot;
  uint32_t carry = 0;
  for (int b0 = 0; b0 < nb; b0 += SCAN_TOP_THREADS) {
    int i = b0 + threadIdx.x;
    uint32_t v = (i < nb) ? block_sums[i] : 0u;
    uint32_t ex = block_excl_scan<SCAN_TOP_THREADS>(v, &tot);
    if (i < nb) block_sums[i] = carry + ex;
    carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    block_sums[nb] = carry;
    if (bump) *step += 1ull;
  }
}

// Phase 3: cell start offsets (exclusive scan), start[n_cells] = total. The
// counts stay: the scatter clears each occupied cell's byte as it reads the
// cell, so the next histogram starts from zero without a pass over all cells.
__global__ void __launch_bounds__(SCAN_THREADS)
    k_scan_apply(const uint32_t *__restrict__ counts, const uint32_t *__restrict__ block_sums,
                 uint32_t *__restrict__ start, int n_cells, int nb) {
  const uint4 q = reinterpret_cast<const uint4 *>(counts)[(size_t)blockIdx.x * SCAN_THREADS +
                                                         threadIdx.x];
  const uint32_t w[4] = {q.x, q.y, q.z, q.w};
  uint32_t v[SCAN_ITEMS];
  uint32_t tsum = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    v[k] = tsum;
    tsum += (w[k >> 2] >> (8 * (k & 3))) & 0xFFu;
  }
  __shared__ uint32_t tot;
  uint32_t off = block_excl_scan<SCAN_THREADS>(tsum, &tot) + block_sums[blockIdx.x];
  uint4 *s4 = reinterpret_cast<uint4 *>(start) + (size_t)blockIdx.x * (SCAN_CHUNK / 4) +
              threadIdx.x * (SCAN_ITEMS / 4);
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS / 4; ++k)
    s4[k] = make_uint4(off + v[4 * k], off + v[4 * k + 1], off + v[4 * k + 2], off + v[4 * k + 3]);
  if (blockIdx.x == 0 && threadIdx.x == 0) start[n_cells] = block_sums[nb];
}

// ------------------------------------------------------------------ scatter

// Counting-sort scatter: bead i goes to slot start[cell] + rank[i] of the
// cell-ordered copy, with its global index packed above the flag bits; the
// slot replaces the rank in rank[i], so the passes that read the pair force
// back in chain order (update, total force) need no cell lookup. The cell's
// byte count is cleared for the next histogram (the scan has consumed it).
__global__ void k_scatter(const Tile *__restrict__ tiles, const SysDesc *__restrict__ sys,
                          const float4 *__restrict__ src, uint32_t *__restrict__ rank,
                          const uint32_t *__restrict__ start, float4 *__restrict__ sorted,
                          float4 *__restrict__ fs_clear, uint32_t *__restrict__ counts,
                          int *__restrict__ err) {
  Tile t = tiles[blockIdx.x];
  const SysDesc &s = sys[t.sys];
  int i = t.begin + threadIdx.x;
  int end = s.bead_off + s.n;
  if (i >= end) return;
  if (fs_clear) fs_clear[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // for the half-shell pass
  bool esc = false;
  float4 p = src[i];
  int c = bead_cell(p, s, esc);
  reinterpret_cast<uint8_t *>(counts)[c] = 0;
  uint32_t slot = start[c] + rank[i];
  if (slot < (uint32_t)s.bead_off || slot >= (uint32_t)end) {
    set_err(err, ERR_SLOT);
    return;
  }
  uint32_t w = ((uint32_t)i << BF_BITS) | (wbits(p) & 7u);
  sorted[slot] = make_float4(p.x, p.y, p.z, __uint_as_float(w));
  rank[i] = slot;
}

// ------------------------------------------------------------------ pair

// Pair term of the warp-per-cell kernel: the coefficient is evaluated for
// every candidate and selected to zero beyond the cutoff or for |i - j| <= 1
// (self included), so the lanes of a warp diverge only between the two
// Lennard-Jones classes (lj_coef). The
// reciprocal is the hardware approximation (<= 2 ulp), well inside the FP32
// force tolerance.
template <int MODE>
__device__ __forceinline__ void pair_accum(float4 p, uint32_t wi, float4 q, const ForceField &ff,
                                           float3 &acc) {
  uint32_t wj = wbits(q);
  int gi = (int)(wi >> BF_BITS), gj = (int)(wj >> BF_BITS);
  bool excl = (unsigned)(gi - gj + 1) <= 2u;
  float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
  float d2 = dx * dx + dy * dy + dz * dz;
  float cf;
  if (MODE == MODE_ICG) {
    float d = sqrtf(d2);
    cf = ff.k_icg * (3.0f * ff.rc_icg - 3.0f * d);
    cf = (excl || d2 > ff.rc_icg * ff.rc_icg) ? 0.0f : cf;
  } else {
    bool hh = (wi & wj & BF_HET) != 0u;
    float rc = hh ? ff.rc_att : ff.rc_rep;
    if (ff.pot == POT_WF) {
      float i2 = __fdividef(1.0f, d2), i4 = i2 * i2;
      cf = 6.0f * ff.e_att * (__fsub_rn(d2, 4.0f) * __fmaf_rn(3.0f, d2, -4.0f)) * (i4 * i4);
    } else {
      cf = hh ? lj_coef<false>(ff.e_att, dx, dy, dz, d2) : lj_coef<true>(ff.e_rep, dx, dy, dz, d2);
    }
    cf = (excl || d2 > rc * rc) ? 0.0f : cf;
  }
  acc.x += cf * dx;
  acc.y += cf * dy;
  acc.z += cf * dz;
}


// Excluded-volume and A-A attraction forces in cell order. Each thread owns
// one sorted bead; for every (dy, dz) row of the 3x3x3 neighbourhood the three
// x-adjacent cells form one contiguous range of the sorted array. Pairs with
// |i - j| <= 1 are skipped, also across chain ends (chrsim.cu:250).
template <int MODE>
__global__ void __launch_bounds__(256)
    k_pair(const Tile *__restrict__ tiles, const SysDesc *__restrict__ sys, ForceField ff,
           const float4 *__restrict__ sorted, const uint32_t *__restrict__ start,
           float4 *__restrict__ fs) {
  Tile t = tiles[blockIdx.x];
  const SysDesc &s = sys[t.sys];
  int slot = t.begin + threadIdx.x;
  if (slot >= s.bead_off + s.n) return;
  float4 p = sorted[slot];
  uint32_t wi = wbits(p);
  bool esc = false;
  CellXYZ c = cell_of(p, s, esc);
  const int cps = s.cps;
  int x0 = max(c.x - 1, 0), x1 = min(c.x + 1, cps - 1);
  float3 acc = make_float3(0.0f, 0.0f, 0.0f);
  for (int z = max(c.z - 1, 0); z <= min(c.z + 1, cps - 1); ++z) {
    for (int y = max(c.y - 1, 0); y <= min(c.y + 1, cps - 1); ++y) {
      int row = s.cell_off + (z * cps + y) * cps;
      uint32_t b = __ldg(&start[row + x0]);
      uint32_t e = __ldg(&start[row + x1 + 1]);
      for (uint32_t k = b; k < e; ++k) {
        float4 q = __ldg(&sorted[k]);
        uint32_t wj = wbits(q);
        int gi = (int)(wi >> BF_BITS), gj = (int)(wj >> BF_BITS);
        float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
        float d2 = dx * dx + dy * dy + dz * dz;
        bool hh = (wi & wj & BF_HET) != 0u;
        float rc = (MODE == MODE_ICG) ? ff.rc_icg : (hh ? ff.rc_att : ff.rc_rep);
        if (d2 > rc * rc || (unsigned)(gi - gj + 1) <= 2u) continue;
        float cf = pair_coef<MODE>(dx, dy, dz, d2, hh, ff);
        acc.x += cf * dx;
        acc.y += cf * dy;
        acc.z += cf * dz;
      }
    }
  }
  fs[slot] = make_float4(acc.x, acc.y, acc.z, 0.0f);
}

// Half-shell pair kernel (Newton's third law). Each sorted bead i visits only
// the forward half of its 27-cell neighbourhood: the beads after it in its own
// cell and the +x cell (one contiguous range), the +y row of the same z layer,
// and the three rows of the +z layer. Every pair is evaluated once; the force
// on i accumulates in registers and the reaction on j is added to fs[j] with a
// vector float4 atomic. fs must be zero on entry (the scatter clears it). Only
// pairs inside the cutoff compute a coefficient and touch memory.
template <int MODE>
__device__ __forceinline__ void half_pair(float4 p, uint32_t wi, const float4 *__restrict__ sorted,
                                          uint32_t k, const ForceField &ff, float3 &acc,
                                          float4 *__restrict__ fs) {
  float4 q = __ldg(&sorted[k]);
  uint32_t wj = wbits(q);
  int gi = (int)(wi >> BF_BITS), gj = (int)(wj >> BF_BITS);
  float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
  float d2 = dx * dx + dy * dy + dz * dz;
  bool hh = (wi & wj & BF_HET) != 0u;
  float rc = (MODE == MODE_ICG) ? ff.rc_icg : (hh ? ff.rc_att : ff.rc_rep);
  if (d2 > rc * rc || (unsigned)(gi - gj + 1) <= 2u) return;
  float cf = pair_coef<MODE>(dx, dy, dz, d2, hh, ff);
  float fx = cf * dx, fy = cf * dy, fz = cf * dz;
  acc.x += fx;
  acc.y += fy;
  acc.z += fz;
  atomicAdd(&fs[k], make_float4(-fx, -fy, -fz, 0.0f));
}

// half_pair on a candidate already loaded, with an early exit for the common
// case: most candidates lie beyond the largest cutoff (rc2_max = its square),
// so the type and chain-neighbour tests run only for the rest.
template <int MODE>
__device__ __forceinline__ void half_pair_q(float4 p, uint32_t wi, float4 q, uint32_t k,
                                            const ForceField &ff, float rc2_max, float3 &acc,
                                            float4 *__restrict__ fs) {
  float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
  float d2 = dx * dx + dy * dy + dz * dz;
  if (d2 > rc2_max) return;
  uint32_t wj = wbits(q);
  bool hh = (wi & wj & BF_HET) != 0u;
  if (MODE != MODE_ICG) {
    float rc = hh ? ff.rc_att : ff.rc_rep;
    if (d2 > rc * rc) return;
  }
  int gi = (int)(wi >> BF_BITS), gj = (int)(wj >> BF_BITS);
  if ((unsigned)(gi - gj + 1) <= 2u) return;
  float cf = pair_coef<MODE>(dx, dy, dz, d2, hh, ff);
  float fx = cf * dx, fy = cf * dy, fz = cf * dz;
  acc.x += fx;
  acc.y += fy;
  acc.z += fz;
  atomicAdd(&fs[k], make_float4(-fx, -fy, -fz, 0.0f));
}

// Candidates [b, e) of one row range, two loads in flight per iteration.
template <int MODE>
__device__ __forceinline__ void half_range(float4 p, uint32_t wi, const float4 *__restrict__ sorted,
                                           uint32_t b, uint32_t e, const ForceField &ff,
                                           float rc2_max, float3 &acc, float4 *__restrict__ fs) {
  uint32_t k = b;
  for (; k + 1 < e; k += 2) {
    float4 q0 = __ldg(&sorted[k]), q1 = __ldg(&sorted[k + 1]);
    half_pair_q<MODE>(p, wi, q0, k, ff, rc2_max, acc, fs);
    half_pair_q<MODE>(p, wi, q1, k + 1, ff, rc2_max, acc, fs);
  }
  if (k < e) half_pair_q<MODE>(p, wi, __ldg(&sorted[k]), k, ff, rc2_max, acc, fs);
}

// REACH = 1: cells of side >= the largest cutoff, 3x3x3 neighbourhood.
// REACH = 2: cells of side >= half of it, 5x5x5 neighbourhood: the candidate
// volume drops from 27 to 15.6 cutoff-cubes (x0.58) at the price of 13 instead
// of 5 row ranges per bead. REACH = 0: each system's own reach (SysDesc), so
// one launch serves systems gridded differently by the autotuner.
template <int MODE, int REACH = 1>
__global__ void __launch_bounds__(256, 8)
    k_pair_half(const Tile *__restrict__ tiles, const SysDesc *__restrict__ sys, ForceField ff,
                const float4 *__restrict__ sorted, const uint32_t *__restrict__ start,
                float4 *__restrict__ fs) {
  Tile t = tiles[blockIdx.x];
  const SysDesc &s = sys[t.sys];
  int slot = t.begin + threadIdx.x;
  if (slot >= s.bead_off + s.n) return;
  const int R = (REACH > 0) ? REACH : s.reach;
  float4 p = sorted[slot];
  uint32_t wi = wbits(p);
  bool esc = false;
  CellXYZ c = cell_of(p, s, esc);
  const int cps = s.cps;
  const int x0 = max(c.x - R, 0), x1 = min(c.x + R, cps - 1);
  const float rc_max = (MODE == MODE_ICG) ? ff.rc_icg : fmaxf(ff.rc_att, ff.rc_rep);
  const float rc2_max = rc_max * rc_max;
  float3 acc = make_float3(0.0f, 0.0f, 0.0f);
  // own cell after i, then the +x cells
  {
    int row = s.cell_off + (c.z * cps + c.y) * cps;
    uint32_t e = __ldg(&start[row + x1 + 1]);
    half_range<MODE>(p, wi, sorted, slot + 1, e, ff, rc2_max, acc, fs);
  }
  // the +y rows of this layer, then all rows of the +z layers
  const int NR = R + R * (2 * R + 1);
#pragma unroll 1
  for (int r = 0; r < NR; ++r) {
    int y, z;
    if (r < R) {
      y = c.y + 1 + r;
      z = c.z;
    } else {
      int q = r - R;
      y = c.y - R + q % (2 * R + 1);
      z = c.z + 1 + q / (2 * R + 1);
    }
    if (y < 0 || y >= cps || z >= cps) continue;
    int row = s.cell_off + (z * cps + y) * cps;
    uint32_t b = __ldg(&start[row + x0]), e = __ldg(&start[row + x1 + 1]);
    half_range<MODE>(p, wi, sorted, b, e, ff, rc2_max, acc, fs);
  }
  atomicAdd(&fs[slot], make_float4(acc.x, acc.y, acc.z, 0.0f));
}

// Pair term of the typed kernel, the pair's class (A-A or not) known from
// the grid it was found in; rc2 = the square of that class's cutoff.
template <int MODE, bool HH>
__device__ __forceinline__ void typed_pair(float4 p, uint32_t wi, float4 q, uint32_t k,
                                           const ForceField &ff, float rc2, float3 &acc,
                                           float4 *__restrict__ fs) {
  float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
  float d2 = dx * dx + dy * dy + dz * dz;
  if (d2 > rc2) return;
  int gi = (int)(wi >> BF_BITS), gj = (int)(wbits(q) >> BF_BITS);
  if ((unsigned)(gi - gj + 1) <= 2u) return;
  float cf = pair_coef<MODE>(dx, dy, dz, d2, HH, ff);
  float fx = cf * dx, fy = cf * dy, fz = cf * dz;
  acc.x += fx;
  acc.y += fy;
  acc.z += fz;
  atomicAdd(&fs[k], make_float4(-fx, -fy, -fz, 0.0f));
}

template <int MODE, bool HH>
__device__ __forceinline__ void typed_range(float4 p, uint32_t wi, const float4 *__restrict__ sorted,
                                            uint32_t b, uint32_t e, const ForceField &ff,
                                            float rc2, float3 &acc, float4 *__restrict__ fs) {
  uint32_t k = b;
  for (; k + 1 < e; k += 2) {
    float4 q0 = __ldg(&sorted[k]), q1 = __ldg(&sorted[k + 1]);
    typed_pair<MODE, HH>(p, wi, q0, k, ff, rc2, acc, fs);
    typed_pair<MODE, HH>(p, wi, q1, k + 1, ff, rc2, acc, fs);
  }
  if (k < e) typed_pair<MODE, HH>(p, wi, __ldg(&sorted[k]), k, ff, rc2, acc, fs);
}

// Forward half of the (2R+1)^3 stencil of cell c in the grid starting at cell
// g0: the beads after `slot` in its own cell and the +x cells, the +y rows of
// its layer, and every row of the +z layers.
template <int MODE, bool HH>
__device__ __forceinline__ void typed_half(float4 p, uint32_t wi, int slot, CellXYZ c, int g0,
                                           int cps, int R, const float4 *__restrict__ sorted,
                                           const uint32_t *__restrict__ start,
                                           const ForceField &ff, float rc2, float3 &acc,
                                           float4 *__restrict__ fs) {
  const int x0 = max(c.x - R, 0), x1 = min(c.x + R, cps - 1);
  {
    int row = g0 + (c.z * cps + c.y) * cps;
    typed_range<MODE, HH>(p, wi, sorted, slot + 1, __ldg(&start[row + x1 + 1]), ff, rc2, acc, fs);
  }
  const int NR = R + R * (2 * R + 1);
#pragma unroll 1
  for (int r = 0; r < NR; ++r) {
    int y, z;
    if (r < R) {
      y = c.y + 1 + r;
      z = c.z;
    } else {
      int q = r - R;
      y = c.y - R + q % (2 * R + 1);
      z = c.z + 1 + q / (2 * R + 1);
    }
    if (y < 0 || y >= cps || z >= cps) continue;
    int row = g0 + (z * cps + y) * cps;
    typed_range<MODE, HH>(p, wi, sorted, __ldg(&start[row + x0]), __ldg(&start[row + x1 + 1]), ff,
                          rc2, acc, fs);
  }
}

// Half-shell pair kernel over the typed layout (SysDesc::cls_cells > 0): in
// every system the A beads are sorted by cell first, then the other beads,
// each class in its own grid. Only A-A pairs interact beyond the repulsive
// cutoff, so
//   an A bead visits A-A pairs over the forward half of the RHH stencil of
//     the A grid and A-other pairs over the full RX stencil of the other grid;
//   another bead visits other-other pairs over the forward half of the RX
//     stencil of the other grid.
// Every unordered pair is visited once, the class of each pair is known from
// its grid, warps hold one class (but at most one per system), and the
// non-A beads scan only the small stencil. RHH / RX = 0: from the system's
// cell side (1 when it is at least the cutoff, else 2).
template <int MODE, int RHH, int RX>
__global__ void __launch_bounds__(256, 8)
    k_pair_typed(const Tile *__restrict__ tiles, const SysDesc *__restrict__ sys, ForceField ff,
                 const float4 *__restrict__ sorted, const uint32_t *__restrict__ start,
                 float4 *__restrict__ fs) {
  Tile t = tiles[blockIdx.x];
  const SysDesc &s = sys[t.sys];
  int slot = t.begin + threadIdx.x;
  if (slot >= s.bead_off + s.n) return;
  float4 p = sorted[slot];
  uint32_t wi = wbits(p);
  bool esc = false;
  CellXYZ c = cell_of(p, s, esc);
  const int cps = s.cps;
  const float rc_hh = (MODE == MODE_ICG) ? ff.rc_icg : ff.rc_att;
  const float rc_x = (MODE == MODE_ICG) ? ff.rc_icg : ff.rc_rep;
  const int rhh = (RHH > 0) ? RHH : (s.csl >= rc_hh ? 1 : 2);
  const int rx = (RX > 0) ? RX : (s.csl >= rc_x ? 1 : 2);
  const int gA = s.cell_off, gX = s.cell_off + s.cls_cells;
  float3 acc = make_float3(0.0f, 0.0f, 0.0f);
  if (wi & BF_HET) {
    typed_half<MODE, true>(p, wi, slot, c, gA, cps, rhh, sorted, start, ff, rc_hh * rc_hh, acc, fs);
    const int x0 = max(c.x - rx, 0), x1 = min(c.x + rx, cps - 1);
    const float rc2 = rc_x * rc_x;
#pragma unroll 1
    for (int z = max(c.z - rx, 0); z <= min(c.z + rx, cps - 1); ++z)
#pragma unroll 1
      for (int y = max(c.y - rx, 0); y <= min(c.y + rx, cps - 1); ++y) {
        int row = gX + (z * cps + y) * cps;
        typed_range<MODE, false>(p, wi, sorted, __ldg(&start[row + x0]),
                                 __ldg(&start[row + x1 + 1]), ff, rc2, acc, fs);
      }
  } else {
    typed_half<MODE, false>(p, wi, slot, c, gX, cps, rx, sorted, start, ff, rc_x * rc_x, acc, fs);
  }
  atomicAdd(&fs[slot], make_float4(acc.x, acc.y, acc.z, 0.0f));
}

// k_pair_half with L lanes per bead (blocks of tile * L threads): the bead's
// row ranges -- its own row and the forward rows -- are dealt round-robin to
// its L lanes, and the lanes' partial forces are combined by shuffles. For
// systems too small to fill the GPU with one thread per bead.
template <int MODE, int REACH, int L>
__global__ void __launch_bounds__(512)
    k_pair_half_lanes(const Tile *__restrict__ tiles, const SysDesc *__restrict__ sys,
                      ForceField ff, const float4 *__restrict__ sorted,
                      const uint32_t *__restrict__ start, float4 *__restrict__ fs) {
  Tile t = tiles[blockIdx.x];
  const SysDesc &s = sys[t.sys];
  const int sub = threadIdx.x % L;
  const int slot = t.begin + threadIdx.x / L;
  const bool valid = slot < s.bead_off + s.n;
  float3 acc = make_float3(0.0f, 0.0f, 0.0f);
  float4 p = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (valid) {
    p = sorted[slot];
    const uint32_t wi = wbits(p);
    bool esc = false;
    CellXYZ c = cell_of(p, s, esc);
    const int cps = s.cps;
    const int x0 = max(c.x - REACH, 0), x1 = min(c.x + REACH, cps - 1);
    const float rc_max = (MODE == MODE_ICG) ? ff.rc_icg : fmaxf(ff.rc_att, ff.rc_rep);
    const float rc2_max = rc_max * rc_max;
    constexpr int NR = REACH + REACH * (2 * REACH + 1);
#pragma unroll 1
    for (int it = sub; it <= NR; it += L) {
      if (it == 0) {  // own cell after i, then the +x cells
        int row = s.cell_off + (c.z * cps + c.y) * cps;
        half_range<MODE>(p, wi, sorted, slot + 1, __ldg(&start[row + x1 + 1]), ff, rc2_max, acc,
                         fs);
        continue;
      }
      const int r = it - 1;
      int y, z;
      if (r < REACH) {
        y = c.y + 1 + r;
        z = c.z;
      } else {
        int q = r - REACH;
        y = c.y - REACH + q % (2 * REACH + 1);
        z = c.z + 1 + q / (2 * REACH + 1);
      }
      if (y < 0 || y >= cps || z >= cps) continue;
      int row = s.cell_off + (z * cps + y) * cps;
      half_range<MODE>(p, wi, sorted, __ldg(&start[row + x0]), __ldg(&start[row + x1 + 1]), ff,
                       rc2_max, acc, fs);
    }
  }
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) {
    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
    acc.z += __shfl_xor_sync(0xffffffffu, acc.z, o);
  }
  if (valid && sub == 0) atomicAdd(&fs[slot], make_float4(acc.x, acc.y, acc.z, 0.0f));
}

// Row (y, z) of forward row r of the half stencil of reach R around c (false
// when it lies outside the grid).
__device__ __forceinline__ bool half_row_yz(CellXYZ c, int r, int R, int cps, int &y, int &z) {
  if (r < R) {
    y = c.y + 1 + r;
    z = c.z;
  } else {
    int q = r - R;
    y = c.y - R + q % (2 * R + 1);
    z = c.z + 1 + q / (2 * R + 1);
  }
  return y >= 0 && y < cps && z < cps;
}

// k_pair_typed with L lanes per bead (blocks of tile * L threads): the bead's
// row ranges are numbered -- own row, forward rows of its grid, then for an A
// bead the rows of the other grid's full stencil -- and dealt round-robin to
// its L lanes; the lanes' partial forces are combined by shuffles.
template <int MODE, int RHH, int RX, int L>
__global__ void __launch_bounds__(512)
    k_pair_typed_lanes(const Tile *__restrict__ tiles, const SysDesc *__restrict__ sys,
                       ForceField ff, const float4 *__restrict__ sorted,
                       const uint32_t *__restrict__ start, float4 *__restrict__ fs) {
  Tile t = tiles[blockIdx.x];
  const SysDesc &s = sys[t.sys];
  const int sub = threadIdx.x % L;
  const int slot = t.begin + threadIdx.x / L;
  const bool valid = slot < s.bead_off + s.n;
  float3 acc = make_float3(0.0f, 0.0f, 0.0f);
  if (valid) {
    const float4 p = sorted[slot];
    const uint32_t wi = wbits(p);
    bool esc = false;
    CellXYZ c = cell_of(p, s, esc);
    const int cps = s.cps;
    const float rc_hh = (MODE == MODE_ICG) ? ff.rc_icg : ff.rc_att;
    const float rc_x = (MODE == MODE_ICG) ? ff.rc_icg : ff.rc_rep;
    const bool isA = (wi & BF_HET) != 0u;
    const int R = isA ? RHH : RX;
    const int g = isA ? s.cell_off : s.cell_off + s.cls_cells;
    const int gX = s.cell_off + s.cls_cells;
    const int NRh = R + R * (2 * R + 1);            // forward rows of the own grid
    const int W = 2 * RX + 1;                        // full stencil rows of the other grid
    const int n_items = 1 + NRh + (isA ? W * W : 0);
    const int x0 = max(c.x - R, 0), x1 = min(c.x + R, cps - 1);
    const int xo0 = max(c.x - RX, 0), xo1 = min(c.x + RX, cps - 1);
#pragma unroll 1
    for (int it = sub; it < n_items; it += L) {
      if (it == 0) {
        int row = g + (c.z * cps + c.y) * cps;
        if (isA)
          typed_range<MODE, true>(p, wi, sorted, slot + 1, __ldg(&start[row + x1 + 1]), ff,
                                  rc_hh * rc_hh, acc, fs);
        else
          typed_range<MODE, false>(p, wi, sorted, slot + 1, __ldg(&start[row + x1 + 1]), ff,
                                   rc_x * rc_x, acc, fs);
      } else if (it <= NRh) {
        int y, z;
        if (!half_row_yz(c, it - 1, R, cps, y, z)) continue;
        int row = g + (z * cps + y) * cps;
        uint32_t b = __ldg(&start[row + x0]), e = __ldg(&start[row + x1 + 1]);
        if (isA)
          typed_range<MODE, true>(p, wi, sorted, b, e, ff, rc_hh * rc_hh, acc, fs);
        else
          typed_range<MODE, false>(p, wi, sorted, b, e, ff, rc_x * rc_x, acc, fs);
      } else {
        const int r = it - 1 - NRh;
        const int y = c.y + r % W - RX, z = c.z + r / W - RX;
        if (y < 0 || y >= cps || z < 0 || z >= cps) continue;
        int row = gX + (z * cps + y) * cps;
        typed_range<MODE, false>(p, wi, sorted, __ldg(&start[row + xo0]),
                                 __ldg(&start[row + xo1 + 1]), ff, rc_x * rc_x, acc, fs);
      }
    }
  }
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) {
    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
    acc.z += __shfl_xor_sync(0xffffffffu, acc.z, o);
  }
  if (valid && sub == 0) atomicAdd(&fs[slot], make_float4(acc.x, acc.y, acc.z, 0.0f));
}

// Half-shell pair kernel with a flattened candidate walk: each lane runs one
// loop over its whole candidate stream and fetches the next row range only
// when the current one is exhausted, so a warp pays the longest total stream
// of its lanes instead of the sum over rows of the longest row.
template <int REACH>
__device__ __forceinline__ void half_row(const SysDesc &s, CellXYZ c, int r, int x0, int x1,
                                         const uint32_t *__restrict__ start, uint32_t &b,
                                         uint32_t &e) {
  int y, z;
  if (r < REACH) {
    y = c.y + 1 + r;
    z = c.z;
  } else {
    int q = r - REACH;
    y = c.y - REACH + q % (2 * REACH + 1);
    z = c.z + 1 + q / (2 * REACH + 1);
  }
  b = e = 0;
  if (y < 0 || y >= s.cps || z >= s.cps) return;
  int row = s.cell_off + (z * s.cps + y) * s.cps;
  b = __ldg(&start[row + x0]);
  e = __ldg(&start[row + x1 + 1]);
}

template <int MODE, int REACH = 1>
__global__ void __launch_bounds__(256)
    k_pair_flat(const Tile *__restrict__ tiles, const SysDesc *__restrict__ sys, ForceField ff,
                const float4 *__restrict__ sorted, const uint32_t *__restrict__ start,
                float4 *__restrict__ fs) {
  Tile t = tiles[blockIdx.x];
  const SysDesc &s = sys[t.sys];
  int slot = t.begin + threadIdx.x;
  if (slot >= s.bead_off + s.n) return;
  float4 p = sorted[slot];
  uint32_t wi = wbits(p);
  bool esc = false;
  CellXYZ c = cell_of(p, s, esc);
  const int cps = s.cps;
  const int x0 = max(c.x - REACH, 0), x1 = min(c.x + REACH, cps - 1);
  constexpr int NR = REACH + REACH * (2 * REACH + 1);
  float3 acc = make_float3(0.0f, 0.0f, 0.0f);
  // range 0: own cell after i and the +x cells
  uint32_t b = slot + 1;
  uint32_t e = __ldg(&start[s.cell_off + (c.z * cps + c.y) * cps + x1 + 1]);
  int r = 0;
  for (;;) {
    while (b >= e) {
      if (r >= NR) goto done;
      half_row<REACH>(s, c, r, x0, x1, start, b, e);
      ++r;
    }
    half_pair<MODE>(p, wi, sorted, b, ff, acc, fs);
    ++b;
  }
done:
  atomicAdd(&fs[slot], make_float4(acc.x, acc.y, acc.z, 0.0f));
}

// Cell-major pair kernel. One warp per cell; the warp's 4 groups of 8 lanes
// each own up to 2 of the cell's beads per pass, and the 8 lanes of a group
// sweep the cell's 27-cell neighbourhood (9 x-contiguous ranges of the sorted
// array, flattened) together. A warp load therefore reads 8 consecutive
// candidates shared by all groups (one 128-byte line), trip counts are uniform
// across the warp, and each candidate feeds two interactions. The group's
// partial forces are combined with 3 shuffle steps. CTA = PAIR_WARPS warps =
// up to PAIR_WARPS consecutive cells of one x-row of one system (tile table).
constexpr int PAIR_WARPS = 8;
constexpr int PAIR_GROUP = 8;                   // lanes per group
constexpr int PAIR_NGROUPS = 32 / PAIR_GROUP;   // groups per warp
constexpr int PAIR_HOME = 2 * PAIR_NGROUPS;     // home beads per warp pass

template <int MODE>
__global__ void __launch_bounds__(PAIR_WARPS * 32, 4)
    k_pair_cells(const Tile *__restrict__ ctiles, const SysDesc *__restrict__ sys, ForceField ff,
                 const float4 *__restrict__ sorted, const uint32_t *__restrict__ start,
                 float4 *__restrict__ fs) {
  // cell starts of the 9 neighbour rows over x in [xb - 1, xb + PAIR_WARPS + 1],
  // staged once for the CTA (all warps reach the barrier before any returns)
  __shared__ uint32_t s_start[9][PAIR_WARPS + 4];
  Tile t = ctiles[blockIdx.x];
  const SysDesc &s = sys[t.sys];
  const int cps = s.cps;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int xb = (t.begin - s.cell_off) % cps, rowi = (t.begin - s.cell_off) / cps;
  const int cy = rowi % cps, cz = rowi / cps;
  for (int idx = threadIdx.x; idx < 9 * (PAIR_WARPS + 4); idx += blockDim.x) {
    int r = idx / (PAIR_WARPS + 4), j = idx % (PAIR_WARPS + 4);
    int y = cy + (r % 3) - 1, z = cz + (r / 3) - 1, xi = xb - 1 + j;
    uint32_t v = 0;
    if (y >= 0 && y < cps && z >= 0 && z < cps && xi >= 0 && xi <= cps)
      v = start[s.cell_off + (z * cps + y) * cps + xi];  // xi = cps: end of the row
    s_start[r][j] = v;
  }
  __syncthreads();
  const int cx = xb + warp;
  if (cx >= cps) return;  // beyond the row segment
  const uint32_t hb = s_start[4][warp + 1], he = s_start[4][warp + 2];
  if (hb == he) return;
  // the 9 candidate ranges (x-adjacent cells of each (dy, dz) row)
  const int j0 = max(cx - 1, 0) - (xb - 1), j1 = min(cx + 1, cps - 1) + 1 - (xb - 1);
  const int g = lane / PAIR_GROUP, gl = lane % PAIR_GROUP;
  for (uint32_t h0 = hb; h0 < he; h0 += PAIR_HOME) {
    const uint32_t ha = h0 + g, hc = h0 + g + PAIR_NGROUPS;
    const bool va = ha < he, vc = hc < he;
    float4 pa = sorted[va ? ha : hb], pc = sorted[vc ? hc : hb];
    uint32_t wa = wbits(pa), wc = wbits(pc);
    float3 aa = make_float3(0.0f, 0.0f, 0.0f), ac = make_float3(0.0f, 0.0f, 0.0f);
    // lane gl visits flattened candidates gl, gl + 8, ...: the offset carried
    // into the next range is where the lane's stride overshot the current one
    uint32_t k = gl;
#pragma unroll
    for (int r = 0; r < 9; ++r) {
      const uint32_t rb = s_start[r][j0], rlen = s_start[r][j1] - rb;
      for (; k < rlen; k += PAIR_GROUP) {
        float4 q = __ldg(&sorted[rb + k]);
        // both home slots are evaluated (an empty slot repeats bead hb and is
        // discarded), so the groups of a warp never diverge
        pair_accum<MODE>(pa, wa, q, ff, aa);
        pair_accum<MODE>(pc, wc, q, ff, ac);
      }
      k -= rlen;
    }
#pragma unroll
    for (int o = PAIR_GROUP / 2; o > 0; o >>= 1) {
      aa.x += __shfl_xor_sync(0xffffffffu, aa.x, o);
      aa.y += __shfl_xor_sync(0xffffffffu, aa.y, o);
      aa.z += __shfl_xor_sync(0xffffffffu, aa.z, o);
      ac.x += __shfl_xor_sync(0xffffffffu, ac.x, o);
      ac.y += __shfl_xor_sync(0xffffffffu, ac.y, o);
      ac.z += __shfl_xor_sync(0xffffffffu, ac.z, o);
    }
    if (gl == 0) {
      if (va) fs[ha] = make_float4(aa.x, aa.y, aa.z, 0.0f);
      if (vc) fs[hc] = make_float4(ac.x, ac.y, ac.z, 0.0f);
    }
  }
}

// ------------------------------------------------------------------ update

// Lamina-binding force on a LAD bead at x (chrsim.cu:202-212, 261-273): sites
// within lco; only cells overlapping [x - lco, x + lco] are visited.
__device__ __forceinline__ float3 lbs_force(float4 x, const SysDesc &s, const ForceField &ff,
                                            const float4 *__restrict__ lbs,
                                            const uint32_t *__restrict__ lbs_start) {
  float3 f = make_float3(0.0f, 0.0f, 0.0f);
  float d = sqrtf(x.x * x.x + x.y * x.y + x.z * x.z);
  float m = ff.lco * 1.001f + 1e-4f;
  if (d < s.lbs_rmin - m || d > s.lbs_rmax + m) return f;  // no site within reach
  bool esc = false;
  int xl = cell_coord(x.x - m, s.inv_csl, s.cps, esc), xh = cell_coord(x.x + m, s.inv_csl, s.cps, esc);
  int yl = cell_coord(x.y - m, s.inv_csl, s.cps, esc), yh = cell_coord(x.y + m, s.inv_csl, s.cps, esc);
  int zl = cell_coord(x.z - m, s.inv_csl, s.cps, esc), zh = cell_coord(x.z + m, s.inv_csl, s.cps, esc);
  const float cl = ff.e_l * (8.0f / (3.0f * ff.lco * ff.lco));
  const float l2h = __fmul_rn(ff.lco, ff.lco), l2l = __fmaf_rn(ff.lco, ff.lco, -l2h);
  for (int z = zl; z <= zh; ++z)
    for (int y = yl; y <= yh; ++y) {
      int row = s.cell_off + (z * s.cps + y) * s.cps;
      uint32_t b = lbs_start[row + xl], e = lbs_start[row + xh + 1];
      for (uint32_t k = b; k < e; ++k) {
        float4 q = lbs[k];
        float vx = x.x - q.x, vy = x.y - q.y, vz = x.z - q.z;
        // (d/lco)^6 - 1 = (n2 - 1)(n2^2 + n2 + 1) with n2 - 1 = (d^2 - lco^2) / lco^2:
        // no cancellation as d -> lco, where the force goes to zero
        float dd = sq3_minus(vx, vy, vz, l2h, l2l);
        if (dd > 0.0f) continue;  // beyond the cutoff
        float m1 = dd / l2h;
        float n2 = 1.0f + m1;
        float cf = cl * m1 * (n2 * n2 + n2 + 1.0f);
        f.x += cf * vx;
        f.y += cf * vy;
        f.z += cf * vz;
      }
    }
  return f;
}

// Bonded (elastic + bending) force on bead i (chrsim.cu:13-76). Bonds exist
// only inside a chain; BF_START marks chain heads. The chain neighbours are
// read through X(j): a chain-order array, or a cell-ordered copy through a
// slot map; the flags are the low bits of each position's w word.
template <class Load>
__device__ __forceinline__ float3 bonded_force_at(Load X, int i, float4 xi, int end,
                                                  const ForceField &ff) {
  uint32_t fi = wbits(xi);
  float4 xm1 = xi, xm2 = xi, xp1 = xi, xp2 = xi;
  bool e1 = (fi & BF_START) == 0u;  // bond (i-1, i)
  bool e0 = false, e2 = false, e3 = false;
  if (e1) {
    xm1 = X(i - 1);
    e0 = (wbits(xm1) & BF_START) == 0u;  // bond (i-2, i-1)
    if (e0) xm2 = X(i - 2);
  }
  if (i + 1 < end) {
    xp1 = X(i + 1);
    e2 = (wbits(xp1) & BF_START) == 0u;  // bond (i, i+1)
    if (e2 && i + 2 < end) {
      xp2 = X(i + 2);
      e3 = (wbits(xp2) & BF_START) == 0u;  // bond (i+1, i+2)
    }
  }
  float3 v0 = e0 ? make_float3(xm1.x - xm2.x, xm1.y - xm2.y, xm1.z - xm2.z) : make_float3(0, 0, 0);
  float3 v1 = e1 ? make_float3(xi.x - xm1.x, xi.y - xm1.y, xi.z - xm1.z) : make_float3(0, 0, 0);
  float3 v2 = e2 ? make_float3(xp1.x - xi.x, xp1.y - xi.y, xp1.z - xi.z) : make_float3(0, 0, 0);
  float3 v3 = e3 ? make_float3(xp2.x - xp1.x, xp2.y - xp1.y, xp2.z - xp1.z) : make_float3(0, 0, 0);
  float il0 = e0 ? rsqrtf(v0.x * v0.x + v0.y * v0.y + v0.z * v0.z) : 0.0f;
  float il1 = e1 ? rsqrtf(v1.x * v1.x + v1.y * v1.y + v1.z * v1.z) : 0.0f;
  float il2 = e2 ? rsqrtf(v2.x * v2.x + v2.y * v2.y + v2.z * v2.z) : 0.0f;
  float il3 = e3 ? rsqrtf(v3.x * v3.x + v3.y * v3.y + v3.z * v3.z) : 0.0f;
  // k_e (1 - l_0 / d) = k_e (d^2 - l_0^2) / ((d + l_0) d), with d^2 - l_0^2 formed
  // from the exact bond vector (rounded difference + its TwoSum residual)
  float lh = __fmul_rn(ff.l_0, ff.l_0), ll = __fmaf_rn(ff.l_0, ff.l_0, -lh);
  float ke1 = 0.0f, ke2 = 0.0f;
  if (e1) {
    float cx = v1.x * two_sum_err(xi.x, -xm1.x, v1.x) + v1.y * two_sum_err(xi.y, -xm1.y, v1.y) +
               v1.z * two_sum_err(xi.z, -xm1.z, v1.z);
    float s1 = __fadd_rn(sq3_minus(v1.x, v1.y, v1.z, lh, ll), 2.0f * cx);
    float d1 = sqrtf(v1.x * v1.x + v1.y * v1.y + v1.z * v1.z);
    ke1 = ff.k_e * (s1 / (d1 + ff.l_0)) * il1;
  }
  if (e2) {
    float cx = v2.x * two_sum_err(xp1.x, -xi.x, v2.x) + v2.y * two_sum_err(xp1.y, -xi.y, v2.y) +
               v2.z * two_sum_err(xp1.z, -xi.z, v2.z);
    float s2 = __fadd_rn(sq3_minus(v2.x, v2.y, v2.z, lh, ll), 2.0f * cx);
    float d2 = sqrtf(v2.x * v2.x + v2.y * v2.y + v2.z * v2.z);
    ke2 = ff.k_e * (s2 / (d2 + ff.l_0)) * il2;
  }
  float3 f = make_float3(ke2 * v2.x - ke1 * v1.x, ke2 * v2.y - ke1 * v1.y, ke2 * v2.z - ke1 * v1.z);
  if (ff.bend_all || (fi & BF_HET)) {
    float cos0 = (v1.x * v0.x + v1.y * v0.y + v1.z * v0.z) * il1 * il0;
    float cos1 = (v2.x * v1.x + v2.y * v1.y + v2.z * v1.z) * il2 * il1;
    float cos2 = (v3.x * v2.x + v3.y * v2.y + v3.z * v2.z) * il3 * il2;
    float a0 = il1 * il0, a1 = il1 * il2, a3 = il2 * il3;
    float i11 = il1 * il1, i22 = il2 * il2;
    // four terms of d/dr_i [cos(theta_{i-1}) + cos(theta_i) + cos(theta_{i+1})]
    float c_v0 = a0;
    float c_v1 = -cos0 * i11 - cos1 * i11 - a1;
    float c_v2 = a1 + cos1 * i22 + cos2 * i22;
    float c_v3 = -a3;
    f.x += ff.k_b * (c_v0 * v0.x + c_v1 * v1.x + c_v2 * v2.x + c_v3 * v3.x);
    f.y += ff.k_b * (c_v0 * v0.y + c_v1 * v1.y + c_v2 * v2.y + c_v3 * v3.y);
    f.z += ff.k_b * (c_v0 * v0.z + c_v1 * v1.z + c_v2 * v2.z + c_v3 * v3.z);
  }
  return f;
}

__device__ __forceinline__ float3 bonded_force(const float4 *__restrict__ X, int i, float4 xi,
                                               int end, const ForceField &ff) {
  return bonded_force_at([X](int j) { return X[j]; }, i, xi, end, ff);
}

// Deterministic displacement of one stage limited to max_step (> 0): keeps the
// stiff WCA core stable at dt = 1e-3 when a truncated-noise jump brings a pair
// deep into it; inactive for |F| dt <= max_step. ccp's preset sets no cap.
__device__ __forceinline__ void cap_step(float3 &D, float max_step) {
  if (max_step <= 0.0f) return;
  float m2 = D.x * D.x + D.y * D.y + D.z * D.z;
  if (m2 > max_step * max_step) {
    float k = max_step * rsqrtf(m2);
    D.x *= k;
    D.y *= k;
    D.z *= k;
  }
}

// Fused chain-order pass of one Heun stage.
//   STAGE 1: X = r.  f = F(r);  er = r + f dt + sd z           (chrsim.cu:365-388)
//   STAGE 2: X = er. ef = F(er); r = r + (f + ef) dt / 2 + sd z (chrsim.cu:392-416)
// F = bonded + wall + LBS + pair (pair read from the cell-ordered result).
// Stage 1 draws the step's noise sd z and keeps it in rnb for stage 2.
// The written position is binned into the next counting sort.
template <int STAGE, int MODE>
__global__ void __launch_bounds__(256, 7)
    k_update(const Tile *__restrict__ tiles, const SysDesc *__restrict__ sys, ForceField ff,
             float4 *__restrict__ pos, float4 *__restrict__ er, float4 *__restrict__ fbuf,
             float4 *__restrict__ rnb, const float4 *__restrict__ fs, uint32_t *__restrict__ rank,
             uint32_t *__restrict__ counts,
             const float4 *__restrict__ lbs, const uint32_t *__restrict__ lbs_start,
             const unsigned long long *__restrict__ step, int *__restrict__ err) {
  Tile t = tiles[blockIdx.x];
  const SysDesc &s = sys[t.sys];
  int i = t.begin + threadIdx.x;
  int end = s.bead_off + s.n;
  if (i >= end) return;
  const float4 *X = (STAGE == 1) ? pos : er;
  float4 xi = X[i];
  uint32_t fl = wbits(xi);

  // pair force of this bead from the cell-ordered pass (its slot, left in
  // rank[i] by the scatter)
  uint32_t slot = rank[i];
  float4 fp = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (slot >= (uint32_t)s.bead_off && slot < (uint32_t)end)
    fp = fs[slot];
  else
    set_err(err, ERR_SLOT);
  float3 F = make_float3(fp.x, fp.y, fp.z);

  float3 fb = bonded_force(X, i, xi, end, ff);
  F.x += fb.x;
  F.y += fb.y;
  F.z += fb.z;

  float3 vw;
  float gh, gl;
  if (wall_vector<MODE>(make_float3(xi.x, xi.y, xi.z), s, vw, gh, gl)) {
    float cw = wall_coef<MODE>(gh, gl, ff);
    F.x += cw * vw.x;
    F.y += cw * vw.y;
    F.z += cw * vw.z;
  }
  if (MODE == MODE_DST && (fl & BF_LAD) && s.n_lbs > 0) {
    float3 fl3 = lbs_force(xi, s, ff, lbs, lbs_start);
    F.x += fl3.x;
    F.y += fl3.y;
    F.z += fl3.z;
  }

  float3 rn = make_float3(0.0f, 0.0f, 0.0f);
  if (MODE == MODE_DST && ff.sd > 0.0f) {
    if (STAGE == 1) {
      float3 z = bead_noise((uint32_t)(i - s.bead_off), *step, s.seed_lo, s.seed_hi, err);
      rn = make_float3(ff.sd * z.x, ff.sd * z.y, ff.sd * z.z);
      rnb[i] = make_float4(rn.x, rn.y, rn.z, 0.0f);
    } else {
      float4 r4 = rnb[i];
      rn = make_float3(r4.x, r4.y, r4.z);
    }
  }

  float4 out;
  if (STAGE == 1) {
    float3 D = make_float3(F.x * ff.dt, F.y * ff.dt, F.z * ff.dt);
    cap_step(D, MODE == MODE_ICG ? ff.icg_max_step : ff.max_step);
    out = make_float4(xi.x + D.x + rn.x, xi.y + D.y + rn.y, xi.z + D.z + rn.z, xi.w);
    er[i] = out;
    fbuf[i] = make_float4(F.x, F.y, F.z, 0.0f);
  } else {
    float4 r = pos[i];
    float4 f1 = fbuf[i];
    float h = 0.5f * ff.dt;
    float3 D = make_float3((f1.x + F.x) * h, (f1.y + F.y) * h, (f1.z + F.z) * h);
    cap_step(D, MODE == MODE_ICG ? ff.icg_max_step : ff.max_step);
    out = make_float4(r.x + D.x + rn.x, r.y + D.y + rn.y, r.z + D.z + rn.z, r.w);
    pos[i] = out;
  }
  if (!(isfinite(out.x) && isfinite(out.y) && isfinite(out.z))) set_err(err, ERR_NAN);
  bool esc2 = false;
  int c_new = bead_cell(out, s, esc2);
  rank[i] = cell_add(counts, c_new, err);
  if (esc2) set_err(err, ERR_ESCAPE);
}

// ------------------------------------------------------------------ forces only

// Total force at the current positions in chain order (for parity checks and
// ccp's host force array): bonded + wall + LBS + pair.
template <int MODE>
__global__ void k_total_force(const Tile *__restrict__ tiles, const SysDesc *__restrict__ sys,
                              ForceField ff, const float4 *__restrict__ pos,
                              const float4 *__restrict__ fs, const uint32_t *__restrict__ rank,
                              const float4 *__restrict__ lbs,
                              const uint32_t *__restrict__ lbs_start, float4 *__restrict__ out) {
  Tile t = tiles[blockIdx.x];
  const SysDesc &s = sys[t.sys];
  int i = t.begin + threadIdx.x;
  int end = s.bead_off + s.n;
  if (i >= end) return;
  float4 xi = pos[i];
  uint32_t slot = rank[i];  // left by the scatter
  float4 fp = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (slot >= (uint32_t)s.bead_off && slot < (uint32_t)end) fp = fs[slot];
  float3 F = make_float3(fp.x, fp.y, fp.z);
  float3 fb = bonded_force(pos, i, xi, end, ff);
  F.x += fb.x;
  F.y += fb.y;
  F.z += fb.z;
  float3 vw;
  float gh, gl;
  if (wall_vector<MODE>(make_float3(xi.x, xi.y, xi.z), s, vw, gh, gl)) {
    float cw = wall_coef<MODE>(gh, gl, ff);
    F.x += cw * vw.x;
    F.y += cw * vw.y;
    F.z += cw * vw.z;
  }
  if (MODE == MODE_DST && (wbits(xi) & BF_LAD) && s.n_lbs > 0) {
    float3 fl3 = lbs_force(xi, s, ff, lbs, lbs_start);
    F.x += fl3.x;
    F.y += fl3.y;
    F.z += fl3.z;
  }
  out[i] = make_float4(F.x, F.y, F.z, 0.0f);
}

// ------------------------------------------------------------------ contacts

// Contact predicate |r_i - r_j| < cutoff with the squared length rounded as
// fma(dz, dz, fma(dx, dx, dy * dy)) and a correctly rounded square root. This
// is the rounding of the reference's compiled length(r[x] - r[y]) < aco
// (chrana.cu:72-73): it reproduces calc_cm on pairs within 4 ulps of the
// cutoff, where the other orderings of the sum do not. Shared with the oracle,
// so counts are bit-exact given identical positions.
__device__ __forceinline__ bool in_contact(float4 a, float4 b, float cut) {
  float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y), dz = __fsub_rn(a.z, b.z);
  float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
  return __fsqrt_rn(d2) < cut;
}

struct ContactArgs {
  float cut;              // contact cutoff (aco = 2 in ccp, chrana.cu:75)
  float mis;              // overlap distance (chrsim.cuh:20)
  int do_map, do_ps, do_overlap;
  int32_t *map;           // packed lower-triangular counts of all systems
  int32_t *ps;            // per-chain contact counts by separation
  const int32_t *chain_of;     // global chain index of every bead
  const int32_t *chain_first;  // first bead of every chain
  const int32_t *chain_ps_off; // offset of every chain in ps
  const int32_t *chain_smax;   // largest separation recorded per chain
  unsigned long long *overlaps;  // per-system overlap count
};



// One unordered pair (i, j) of the half-shell contact pass, in either order:
// the pair is counted for the bead with the lower index, as the full-stencil
// pass counts it (gj > gi).
struct ContactBead {
  int g, copy, lc, bin, ch;
  bool mapped;
};

__device__ __forceinline__ ContactBead contact_bead(int g, const SysDesc &s, const ContactArgs &a) {
  ContactBead b;
  b.g = g;
  int l = g - s.bead_off;
  b.copy = l / s.copy_len;
  b.lc = l - b.copy * s.copy_len;
  b.mapped = b.copy < s.n_copies && b.lc < s.map_len;
  b.bin = b.mapped ? (int)(((long long)b.lc * s.nbins) / s.map_len) : 0;
  b.ch = a.chain_of[g];
  return b;
}

__device__ __forceinline__ void contact_pair(float4 p, const ContactBead &bi, float4 q,
                                             const SysDesc &s, const ContactArgs &a,
                                             unsigned long long &novl) {
  int gj = (int)(wbits(q) >> BF_BITS);
  int lo = min(bi.g, gj), hi = max(bi.g, gj);
  if (a.do_overlap && hi - lo >= 2 && in_contact(p, q, a.mis)) ++novl;
  if (!in_contact(p, q, a.cut)) return;
  ContactBead bj = contact_bead(gj, s, a);
  if (a.do_map && bi.mapped && bj.mapped && bi.copy == bj.copy) {
    int bx = max(bi.bin, bj.bin), by = min(bi.bin, bj.bin);
    long long idx = s.map_off + (long long)bx * (bx + 1) / 2 + by;
    atomicAdd(&a.map[idx], bx == by ? 2 : 1);
  }
  if (a.do_ps && bj.ch == bi.ch) {
    int sep = hi - lo;
    if (sep <= a.chain_smax[bi.ch]) atomicAdd(&a.ps[a.chain_ps_off[bi.ch] + sep], 1);
  }
}

// Forward half of the (2R+1)^3 stencil in the grid starting at cell g0 (the
// own cell after `slot` and the +x cells, the +y rows, the +z layers), or
// the full stencil (FULL) of that grid.
template <bool FULL>
__device__ __forceinline__ void contact_rows(float4 p, const ContactBead &bi, int slot, CellXYZ c,
                                             int g0, int R, const SysDesc &s,
                                             const float4 *__restrict__ sorted,
                                             const uint32_t *__restrict__ start,
                                             const ContactArgs &a, unsigned long long &novl) {
  const int cps = s.cps;
  const int x0 = max(c.x - R, 0), x1 = min(c.x + R, cps - 1);
  if (FULL) {
    for (int z = max(c.z - R, 0); z <= min(c.z + R, cps - 1); ++z)
      for (int y = max(c.y - R, 0); y <= min(c.y + R, cps - 1); ++y) {
        int row = g0 + (z * cps + y) * cps;
        for (uint32_t k = __ldg(&start[row + x0]), e = __ldg(&start[row + x1 + 1]); k < e; ++k)
          contact_pair(p, bi, __ldg(&sorted[k]), s, a, novl);
      }
    return;
  }
  {
    int row = g0 + (c.z * cps + c.y) * cps;
    for (uint32_t k = slot + 1, e = __ldg(&start[row + x1 + 1]); k < e; ++k)
      contact_pair(p, bi, __ldg(&sorted[k]), s, a, novl);
  }
  const int NR = R + R * (2 * R + 1);
  for (int r = 0; r < NR; ++r) {
    int y, z;
    if (r < R) {
      y = c.y + 1 + r;
      z = c.z;
    } else {
      int q = r - R;
      y = c.y - R + q % (2 * R + 1);
      z = c.z + 1 + q / (2 * R + 1);
    }
    if (y < 0 || y >= cps || z >= cps) continue;
    int row = g0 + (z * cps + y) * cps;
    for (uint32_t k = __ldg(&start[row + x0]), e = __ldg(&start[row + x1 + 1]); k < e; ++k)
      contact_pair(p, bi, __ldg(&sorted[k]), s, a, novl);
  }
}

// One pass over unordered bead pairs within the contact cutoff of the
// cell-ordered copy: binned contact map (calc_cm, chrana.cu:48-84), per-chain
// contact counts by separation (the cp part of calc_sd_cp, chrana.cu:13-45) and
// the overlap count of the initial-condition relaxation (chrsim.cu:805-820).
// Every unordered pair is visited once, over half stencils: one grid, or the
// typed layout's A-A half, A-other full and other-other half stencils (the
// contact predicate is symmetric in i and j). REACH as for the pair kernel
// (cells of side >= cutoff / REACH); 0: each system's own reach.
template <int REACH = 1>
__global__ void __launch_bounds__(256)
    k_contacts_half(const Tile *__restrict__ tiles, const SysDesc *__restrict__ sys,
                    const float4 *__restrict__ sorted, const uint32_t *__restrict__ start,
                    ContactArgs a) {
  Tile t = tiles[blockIdx.x];
  const SysDesc &s = sys[t.sys];
  int slot = t.begin + threadIdx.x;
  unsigned long long novl = 0;
  if (slot < s.bead_off + s.n) {
    float4 p = sorted[slot];
    ContactBead bi = contact_bead((int)(wbits(p) >> BF_BITS), s, a);
    bi.mapped = bi.mapped && a.do_map;
    bool esc = false;
    CellXYZ c = cell_of(p, s, esc);
    const int R = (REACH > 0) ? REACH : s.reach;
    if (s.cls_cells == 0) {
      contact_rows<false>(p, bi, slot, c, s.cell_off, R, s, sorted, start, a, novl);
    } else if (wbits(p) & BF_HET) {
      contact_rows<false>(p, bi, slot, c, s.cell_off, R, s, sorted, start, a, novl);
      contact_rows<true>(p, bi, slot, c, s.cell_off + s.cls_cells, R, s, sorted, start, a, novl);
    } else {
      contact_rows<false>(p, bi, slot, c, s.cell_off + s.cls_cells, R, s, sorted, start, a, novl);
    }
  }
  if (a.do_overlap) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) novl += __shfl_xor_sync(0xffffffffu, novl, o);
    if ((threadIdx.x & 31) == 0 && novl) atomicAdd(&a.overlaps[t.sys], novl);
  }
}

// ------------------------------------------------------------------ observables

constexpr int N_SHELLS = 64;  // radial bins (chrana.cuh:16)

// Per-system FP64 accumulators: [0..2] sum r, [3] sum |r|^2, then 3 x 64 radial
// density volumes (A, B, all) of chrana.cu:422-480.
constexpr int OBS_STRIDE = 4 + 3 * N_SHELLS;

// Each warp accumulates the shell volumes of its 32 beads in its own FP32
// shared histogram (native shared float atomics; a bead near the wall spans up
// to ~20 thin outer shells); the position sums for Rg^2 are reduced in FP64 by
// warp shuffles. The CTA then folds the warp histograms into FP64 and adds the
// non-zero entries to the system's accumulators.
constexpr int OBS_WARPS = 8;  // most warps of a CTA (tiles of up to 256 beads)

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(OBS_WARPS * 32)
    k_observe(const Tile *__restrict__ tiles, const SysDesc *__restrict__ sys,
              const float4 *__restrict__ pos, float bead_r, double *__restrict__ acc) {
  __shared__ float hist[OBS_WARPS][3 * N_SHELLS];
  __shared__ double sums[4];
  __shared__ float rb[N_SHELLS];
  Tile t = tiles[blockIdx.x];
  const SysDesc &s = sys[t.sys];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int k = threadIdx.x; k < OBS_WARPS * 3 * N_SHELLS; k += blockDim.x) (&hist[0][0])[k] = 0.0f;
  if (threadIdx.x < 4) sums[threadIdx.x] = 0.0;
  for (int k = threadIdx.x; k < N_SHELLS; k += blockDim.x)
    rb[k] = s.R_n * cbrtf((k + 1.0f) / N_SHELLS);
  __syncthreads();
  int i = t.begin + threadIdx.x;
  double px = 0.0, py = 0.0, pz = 0.0;
  if (i < s.bead_off + s.n) {
    float4 p = pos[i];
    bool het = (wbits(p) & BF_HET) != 0u;
    px = p.x;
    py = p.y;
    pz = p.z;
    float dr = sqrtf(p.x * p.x + p.y * p.y + p.z * p.z);
    const float a = bead_r;
    const float vfull = (4.0f / 3.0f) * 3.14159265358979f * a * a * a;
    // first shell that can overlap the bead (a few below the estimate)
    float inner = fmaxf(dr - a, 0.0f) / s.R_n;
    int b0 = max(0, (int)floorf(N_SHELLS * inner * inner * inner) - 2);
    float vprev = 0.0f;
    float *h = hist[warp];
    for (int b = b0; b < N_SHELLS; ++b) {
      float r = rb[b], v;
      if (dr - a > r) {
        v = 0.0f;
      } else if (dr + a < r) {
        v = vfull;
      } else {
        float ca = (dr * dr + a * a - r * r) / (2.0f * dr * a);
        float cb = (r * r + dr * dr - a * a) / (2.0f * r * dr);
        float va = (3.14159265358979f / 3.0f) * a * a * a * (2.0f + ca) * (1.0f - ca) * (1.0f - ca);
        float vb = (3.14159265358979f / 3.0f) * r * r * r * (2.0f + cb) * (1.0f - cb) * (1.0f - cb);
        v = va + vb;
      }
      float dv = v - vprev;
      vprev = v;
      if (dv != 0.0f) {
        atomicAdd(&h[(het ? 0 : 1) * N_SHELLS + b], dv);
        atomicAdd(&h[2 * N_SHELLS + b], dv);
      }
      if (dr + a < r) break;  // bead inside shell b: all further shells get zero
    }
  }
  double sx = warp_sum_d(px), sy = warp_sum_d(py), sz = warp_sum_d(pz);
  double sr = warp_sum_d(px * px + py * py + pz * pz);
  if (lane == 0) {
    atomicAdd(&sums[0], sx);
    atomicAdd(&sums[1], sy);
    atomicAdd(&sums[2], sz);
    atomicAdd(&sums[3], sr);
  }
  __syncthreads();
  double *dst = acc + (size_t)t.sys * OBS_STRIDE;
  if (threadIdx.x < 4 && sums[threadIdx.x] != 0.0) atomicAdd(&dst[threadIdx.x], sums[threadIdx.x]);
  for (int k = threadIdx.x; k < 3 * N_SHELLS; k += blockDim.x) {
    double v = 0.0;
#pragma unroll
    for (int w = 0; w < OBS_WARPS; ++w)
      if (w < (int)(blockDim.x >> 5)) v += (double)hist[w][k];
    if (v != 0.0) atomicAdd(&dst[4 + k], v);
  }
}

// Per-frame nematic order parameter and nucleus chromatin fraction sums of
// every system (chrana.cu:396-418): fx[2 s] += over beads i < n - 1 of the
// system (3 cos^2 - 1) / 2, cos the angle between the bond i -> i + 1 and
// r_i (over chain ends too, as ccp); fx[2 s + 1] += beads with z < nod. FP64.
__global__ void __launch_bounds__(256)
    k_frame_extra(const Tile *__restrict__ tiles, const SysDesc *__restrict__ sys,
                  const float4 *__restrict__ pos, double *__restrict__ fx) {
  Tile t = tiles[blockIdx.x];
  const SysDesc &s = sys[t.sys];
  const int i = t.begin + threadIdx.x;
  const int end = s.bead_off + s.n;
  double nop = 0.0, ncf = 0.0;
  if (i < end) {
    const float4 p = pos[i];
    if (p.z < s.nod) ncf = 1.0;
    if (i + 1 < end) {
      const float4 q = pos[i + 1];
      const double bx = (double)q.x - p.x, by = (double)q.y - p.y, bz = (double)q.z - p.z;
      const double c = (bx * p.x + by * p.y + bz * p.z) /
                       (sqrt(bx * bx + by * by + bz * bz) *
                        sqrt((double)p.x * p.x + (double)p.y * p.y + (double)p.z * p.z));
      nop = 0.5 * (3.0 * c * c - 1.0);
    }
  }
  nop = warp_sum_d(nop);
  ncf = warp_sum_d(ncf);
  if ((threadIdx.x & 31) == 0) {
    if (nop != 0.0) atomicAdd(&fx[2 * t.sys], nop);
    if (ncf != 0.0) atomicAdd(&fx[2 * t.sys + 1], ncf);
  }
}

// Mean spatial distance by separation (the sd part of calc_sd_cp,
// chrana.cu:13-45): ds[chain_ps_off + s] += sum_p |r_{p+s} - r_p| over a chunk
// of p, FP32 distances accumulated in FP64.
constexpr int SDIST_PCHUNK = 256;

__global__ void __launch_bounds__(256)
    k_sdist(const float4 *__restrict__ pos, const int32_t *__restrict__ chain_first,
            const int32_t *__restrict__ chain_len, const int32_t *__restrict__ chain_ps_off,
            const int32_t *__restrict__ chain_smax, int chain, double *__restrict__ ds) {
  int first = chain_first[chain], L = chain_len[chain], smax = chain_smax[chain];
  int sep = blockIdx.x * blockDim.x + threadIdx.x + 1;
  int p0 = blockIdx.y * SDIST_PCHUNK;
  if (sep > smax || p0 >= L - sep) return;
  int p1 = min(p0 + SDIST_PCHUNK, L - sep);
  float acc = 0.0f;
  for (int p = p0; p < p1; ++p) {
    float4 a = pos[first + p], b = pos[first + p + sep];
    float dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
    acc += sqrtf(dx * dx + dy * dy + dz * dz);
  }
  atomicAdd(&ds[chain_ps_off[chain] + sep], (double)acc);
}

// Sets the device step counter (the first scan of the next step bumps it).
__global__ void k_set_step(unsigned long long *step, unsigned long long v) { *step = v; }

// ------------------------------------------------ initial condition: random walk

// One chain of the confined random walk (chrsim::perform_random_walk,
// chrsim.cu:719-802).
struct WalkChain {
  int32_t first, end;    // beads [first, end) of pos
  uint32_t k0, k1;       // Philox key: the system's seed
  uint32_t chain;        // chain index within its system (the stream)
  uint32_t max_draws;    // draw budget of the chain
  double ax, ay, az;     // cone axis; zero: no cone
  double cos_mda;        // cosine of the cone half-angle
  double R_n;            // nucleus radius
};

// Constants of the walk shared by every chain.
struct WalkParams {
  double inv_cb;   // 1 / c_b, c_b = 0.5 k_b / kT: cos(bond angle) has density exp(c_b cos)
  double one_m_e;  // 1 - exp(-2 c_b)
  double l_0;      // rest bond length
  double sig_b;    // sqrt(2 kT / k_e): bond-length spread
  double mis;      // smallest allowed distance to the wall
};

// Draw d of a chain: one Philox block per attempt (two uniforms for the random
// direction, one for the bond angle, one for the bond length).
__device__ __forceinline__ U32x4 walk_bits(const WalkChain &w, uint32_t d) {
  U32x4 c{d, w.chain, (STREAM_INIT << 16) | 0x57u, 0x1C0DEu};
  return philox4x32_10(c, w.k0, w.k1);
}

__device__ __forceinline__ double walk_u(uint32_t x) {
  return (double)((x >> 8) + 1u) * (1.0 / 16777216.0);  // (0, 1], 24 bits
}

// Uniform direction on the sphere from two (0, 1] uniforms:
// cos(theta) = 1 - 2 u, phi = 2 pi v.
__device__ __forceinline__ double3 walk_direction(uint32_t a, uint32_t b) {
  double ct = 1.0 - 2.0 * walk_u(a);
  double st = sqrt(fmax(0.0, 1.0 - ct * ct));
  double sp, cp;
  sincospi(2.0 * walk_u(b), &sp, &cp);
  return make_double3(st * cp, st * sp, ct);
}

// Cone test of the reference, acos(r.a / (|r| |a|)) > mda rejects, written
// without the arc cosine and the division: r.a < cos(mda) |r| |a| rejects (a
// NaN passes, as in the reference's comparison); a zero axis has no cone.
__device__ __forceinline__ bool walk_in_cone(const WalkChain &w, double la, double3 p, double dr) {
  if (la == 0.0) return true;
  return !((p.x * w.ax + p.y * w.ay + p.z * w.az) < w.cos_mda * dr * la);
}

// One warp per chain, in FP64 (the walk is latency-bound; FP64 makes it
// reproducible to rounding by a CPU restatement, decision for decision). The
// walk is the reference's sequential rejection walk: attempts for a bead
// continue until one is accepted (finite, at least mis from the wall, inside
// the cone); after more than 1024 consecutive rejections every further
// rejection moves to bead first + 2 + (i - first) * 3 / 4, continuing from the
// position stored there (the last rejected candidate of a bead stays stored,
// as in the reference). Lanes evaluate consecutive attempts of the same bead
// at once -- attempt k of the chain always uses draw k -- and the lowest
// accepted lane is the attempt the sequential walk accepts; a chunk never
// extends past the attempt that triggers a move back. So the walk equals the
// sequential one. Chunks start at one attempt and double after each chunk
// that is rejected whole (up to 32), so a walk that is mostly accepted keeps
// one lane busy. wxyz holds the FP64 positions the walk continues from; pos
// receives them in FP32. A chain that exceeds its draw budget sets ERR_WALK.
constexpr int WALK_WARPS = 4;

__global__ void __launch_bounds__(32 * WALK_WARPS)
k_random_walk(const WalkChain *__restrict__ chains, int n_chains, WalkParams wp,
              float4 *__restrict__ pos, double *__restrict__ wxyz,
              uint32_t *__restrict__ draws_used, int *__restrict__ err) {
  const int lane = threadIdx.x & 31;
  const int c = blockIdx.x * WALK_WARPS + (threadIdx.x >> 5);
  if (c >= n_chains) return;
  const WalkChain w = chains[c];
  const double la = sqrt(w.ax * w.ax + w.ay * w.ay + w.az * w.az);
  const double r_in = w.R_n - wp.mis;
  const unsigned FULL = 0xFFFFFFFFu;
  uint32_t draw = 0;
  int chunk = 1;
  double3 old, prev;
  // first bead: radial distance (R_n - mis) u^(1/3) along a random direction
  for (;;) {
    if (draw + (uint32_t)chunk > w.max_draws) {
      if (lane == 0) {
        set_err(err, ERR_WALK);
        draws_used[c] = draw;
      }
      return;
    }
    double3 d = make_double3(0.0, 0.0, 0.0), p = d;
    bool ok = false;
    if (lane < chunk) {
      U32x4 r = walk_bits(w, draw + lane);
      d = walk_direction(r.x, r.y);
      double dr = r_in * cbrt(walk_u(r.z));
      p = make_double3(dr * d.x, dr * d.y, dr * d.z);
      ok = walk_in_cone(w, la, p, dr);
    }
    unsigned acc = __ballot_sync(FULL, ok);
    if (acc) {
      int j = __ffs(acc) - 1;
      old = make_double3(__shfl_sync(FULL, d.x, j), __shfl_sync(FULL, d.y, j),
                         __shfl_sync(FULL, d.z, j));
      prev = make_double3(__shfl_sync(FULL, p.x, j), __shfl_sync(FULL, p.y, j),
                          __shfl_sync(FULL, p.z, j));
      draw += (uint32_t)j + 1u;
      if (lane == 0) {
        float4 v = pos[w.first];
        pos[w.first] = make_float4((float)prev.x, (float)prev.y, (float)prev.z, v.w);
        double *q = wxyz + 3 * (size_t)w.first;
        q[0] = prev.x;
        q[1] = prev.y;
        q[2] = prev.z;
      }
      break;
    }
    draw += (uint32_t)chunk;
    chunk = min(2 * chunk, 32);
  }
  int att = 0;
  int i = w.first + 1;
  chunk = 1;
  while (i < w.end) {
    const int m = (att >= 1024) ? 1 : min(chunk, 1025 - att);
    if (draw + (uint32_t)m > w.max_draws) {
      if (lane == 0) set_err(err, ERR_WALK);
      break;
    }
    double3 p = prev, nd = old;
    bool ok = false;
    if (lane < m) {
      U32x4 r = walk_bits(w, draw + lane);
      double3 rd = walk_direction(r.x, r.y);
      double3 per = make_double3(old.y * rd.z - old.z * rd.y, old.z * rd.x - old.x * rd.z,
                                 old.x * rd.y - old.y * rd.x);
      double il = rsqrt(per.x * per.x + per.y * per.y + per.z * per.z);
      // cos of the bond angle by inversion of its density exp(c_b cos) on [-1, 1]
      double cb = 1.0 + log1p(-wp.one_m_e * walk_u(r.z)) * wp.inv_cb;
      if (cb > 1.0) cb = 1.0;  // comparisons keep a NaN (rejected, like acos(NaN))
      if (cb < -1.0) cb = -1.0;
      double sb = sqrt(1.0 - cb * cb) * il;
      nd = make_double3(cb * old.x + sb * per.x, cb * old.y + sb * per.y, cb * old.z + sb * per.z);
      double lb = wp.l_0 + wp.sig_b * erfinv(2.0 * walk_u(r.w) - 1.0);
      p = make_double3(lb * nd.x + prev.x, lb * nd.y + prev.y, lb * nd.z + prev.z);
      double dr = sqrt(p.x * p.x + p.y * p.y + p.z * p.z);
      ok = isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && !((w.R_n - dr) < wp.mis) &&
           walk_in_cone(w, la, p, dr);
    }
    unsigned acc = __ballot_sync(FULL, ok);
    // the accepted candidate, or the last rejected one, stays stored at bead i
    const int j = acc ? __ffs(acc) - 1 : m - 1;
    if (lane == j) {
      float4 v = pos[i];
      pos[i] = make_float4((float)p.x, (float)p.y, (float)p.z, v.w);
      double *q = wxyz + 3 * (size_t)i;
      q[0] = p.x;
      q[1] = p.y;
      q[2] = p.z;
    }
    if (acc) {
      old = make_double3(__shfl_sync(FULL, nd.x, j), __shfl_sync(FULL, nd.y, j),
                         __shfl_sync(FULL, nd.z, j));
      prev = make_double3(__shfl_sync(FULL, p.x, j), __shfl_sync(FULL, p.y, j),
                          __shfl_sync(FULL, p.z, j));
      draw += (uint32_t)j + 1u;
      att = 0;
      chunk = 1;
      ++i;
    } else {
      draw += (uint32_t)m;
      att = min(att + m, 1 << 20);  // only att > 1024 matters
      chunk = min(2 * chunk, 32);
      if (att > 1024) {
        i = w.first + 2 + (i - w.first) * 3 / 4;
        __syncwarp();
        const double *q = wxyz + 3 * (size_t)(i - 1);
        prev = make_double3(q[0], q[1], q[2]);
      }
    }
  }
  if (lane == 0) draws_used[c] = draw;
}

// Packed xyz triples written into the positions, keeping each bead's flags.
__global__ void k_unpack_xyz(const float *__restrict__ xyz, float4 *__restrict__ pos, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float w = pos[i].w;
  pos[i] = make_float4(xyz[3 * i + 0], xyz[3 * i + 1], xyz[3 * i + 2], w);
}

// Positions as packed xyz triples (the .trr / checkpoint layout).
__global__ void k_pack_xyz(const float4 *__restrict__ pos, float *__restrict__ xyz, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p = pos[i];
  xyz[3 * i + 0] = p.x;
  xyz[3 * i + 1] = p.y;
  xyz[3 * i + 2] = p.z;
}

}  // namespace ccpgpu
