// Shared host/device definitions of the GB300 Brownian-dynamics engine for the
// ccp chromatin model: bead flags, the per-system descriptor, the runtime force
// field, Philox4x32-10 and the truncated Box-Muller noise.
//
// Reference correspondences (Marco-Mendivil-Carboni/TFM, Program/src):
//   model constants        chrdat.cuh:15-24, chrsim.cuh:18-20
//   nucleus geometry       chrdat.cu:13-18 (cngeom)
//   bead types A/B         chrdat.cuh:40-44 (LADh / LNDe)
//   noise and truncation   chrsim.cu:336-361 (begin_iter)
#pragma once

#include <cstdint>

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif

namespace ccpgpu {

// ---------------------------------------------------------------- bead flags
// Stored in the w word of every float4 position (bit pattern, never used as a
// float). In the cell-sorted copy the bead's global index sits above the flags.
enum : uint32_t {
  BF_HET = 1u,    // type A (LADh, heterochromatin-like): A-A attraction
  BF_LAD = 2u,    // binds lamina-binding sites
  BF_START = 4u,  // first bead of a chain: no bond to the previous bead
  BF_BITS = 3u,   // number of flag bits below the index in sorted words
};

// ---------------------------------------------------------------- force field
enum : int {
  POT_WF = 0,  // Wang-Frenkel, rc = 2 form (ccp, chrsim.cu:174-185)
  POT_LJ = 1,  // Lennard-Jones (WCA repulsion + A-A attraction)
};

enum : int {
  MODE_DST = 0,  // production dynamics (chrsim.cuh:29 DST)
  MODE_ICG = 1,  // initial-condition relaxation (chrsim.cuh:30 ICG)
};

struct ForceField {
  int pot;          // POT_WF or POT_LJ (pair and wall form)
  int bend_all;     // 1: bending on every bead; 0: only on BF_HET beads (ccp)
  float k_e, l_0;   // harmonic bond
  float k_b;        // cosine bending
  float e_att;      // A-A pair energy (WF epsilon / LJ epsilon)
  float e_rep;      // LJ epsilon of the purely repulsive (non A-A) pairs
  float rc_rep;     // repulsive cutoff (WF minimum 2/sqrt(3), or 2^(1/6))
  float rc_att;     // A-A cutoff (WF 2, LJ 2.5)
  float e_w, rc_w;  // wall energy and cutoff (distance to the wall)
  float e_l, lco;   // lamina-binding energy and cutoff
  float lbs_depth;  // LBS sit at R_n - lbs_depth
  float k_icg;      // soft repulsion of the ICG mode (128)
  float rc_icg;     // soft repulsion cutoff (rco)
  float mis;        // relaxation ends when no non-bonded pair is closer (chrsim.cuh:20)
  float max_step;   // cap on the deterministic displacement of one stage (0: none)
  float dt;         // time step
  float sd;         // noise standard deviation sqrt(2 kT dt)
  float kT;         // thermal energy
  float icg_max_step;  // the same cap for the relaxation steps (MODE_ICG)
};

// ---------------------------------------------------------------- systems
// One independent replica: a confined polymer with its own cell grid, LBS,
// seed and contact map. A ccp run is a batch of one system.
struct SysDesc {
  int32_t bead_off, n;       // beads [bead_off, bead_off + n), chain order
  int32_t cell_off, cps;     // cps^3 cells starting at cell_off
  float csl, inv_csl;        // cell side length and its inverse
  float R_n, R_o, R_b;       // nucleus, opening and bleb radii
  float noc, boc, nod, bod;  // derived geometry (chrdat.cu:13-18)
  int32_t lbs_off, n_lbs;    // LBS, sorted by cell, [lbs_off, lbs_off + n_lbs)
  float lbs_rmin, lbs_rmax;  // radial extent of the system's LBS
  uint32_t seed_lo, seed_hi; // Philox key
  int32_t chain_off, n_chains;
  // contact map (packed lower triangle of nbins x nbins int32 counts)
  int64_t map_off;
  int32_t nbins, map_len, copy_len, n_copies;
  int32_t sys_index;
  int32_t reach;  // neighbour cells per axis (1: csl >= cutoff, 2: csl >= cutoff / 2)
  // typed layout: the cells of the non-A beads start cls_cells after those of
  // the A beads (cps^3); 0: one grid for all beads
  int32_t cls_cells;
};

// ---------------------------------------------------------------- Philox
struct U32x4 {
  uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ void mulhilo32(uint32_t a, uint32_t b,
                                                   uint32_t &hi, uint32_t &lo) {
#ifdef __CUDA_ARCH__
  lo = a * b;
  hi = __umulhi(a, b);
#else
  uint64_t p = (uint64_t)a * (uint64_t)b;
  lo = (uint32_t)p;
  hi = (uint32_t)(p >> 32);
#endif
}

// Philox4x32 with 10 rounds (Salmon, Moraes, Dror, Shaw; SC'11).
__host__ __device__ __forceinline__ U32x4 philox4x32_10(U32x4 c, uint32_t k0,
                                                        uint32_t k1) {
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(0xD2511F53u, c.x, hi0, lo0);
    mulhilo32(0xCD9E8D57u, c.z, hi1, lo1);
    c = U32x4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

// Counter layout of the dynamics noise: (bead index within its system,
// attempt | stream << 16, step low word, step high word); key = system seed.
// A system therefore draws the same noise whether it runs alone or batched.
enum : uint32_t { STREAM_BD = 0u, STREAM_INIT = 1u };

__host__ __device__ __forceinline__ U32x4 noise_bits(uint32_t bead,
                                                     uint32_t attempt,
                                                     uint64_t step,
                                                     uint32_t k0, uint32_t k1) {
  U32x4 c{bead, attempt | (STREAM_BD << 16), (uint32_t)step,
          (uint32_t)(step >> 32)};
  return philox4x32_10(c, k0, k1);
}

// Uniforms for Box-Muller built from the top 24 bits so that they are exact
// in float: u1 in (0, 1], u2 in [0, 1).
__host__ __device__ __forceinline__ float u01_open0(uint32_t x) {
  return (float)((x >> 8) + 1u) * (1.0f / 16777216.0f);
}
__host__ __device__ __forceinline__ float u01_open1(uint32_t x) {
  return (float)(x >> 8) * (1.0f / 16777216.0f);
}

// The relaxation (ICG) wall is ccp's Wang-Frenkel wall with eps = 1 and cutoff
// rco for every preset (calc_cf<ICG>, chrsim.cu:148-170).
constexpr float ICG_WALL_RC = 1.154701f;

constexpr int NOISE_MAX_ATTEMPTS = 64;
constexpr float NOISE_TRUNC = 5.0f;  // |z| <= 5 (chrsim.cu:356)

}  // namespace ccpgpu
