// Persistent per-system Heun stepping in shared memory.
//
// One CTA owns one system and advances it by `nsteps` stochastic Heun steps
// (chrsim.cu:365-416) in a single launch, with every array of the step in
// its shared memory: positions, the cell-ordered copy and its cell starts,
// the pair forces, the stage-1 force. Phases are separated by __syncthreads
// only, so a frame of steps costs one launch instead of twelve per step;
// that is what bounds small systems (a 2048-bead chain spends most of a
// graph-launched Heun step waiting on launches on 16 of 152 SMs). A batch
// runs one CTA per system, so a batch of small systems is one launch per
// frame.
//
// Per bead and step it computes what the graph path's kernels do, term for
// term and with the same helpers: the cell-list counting sort (sugrid.cu,
// replaced by a shared-memory histogram, scan and scatter), the half-shell
// pair pass (chrsim.cu:224-317), bonded + bending (chrsim.cu:13-76), wall
// (chrsim.cu:79-170), lamina binding (chrsim.cu:202-220; sites read from the
// system's static global grid), the counter-based noise of the same Philox
// stream (so a system draws the same noise on either path) and the
// displacement cap. Only the FP32 summation order of the pair forces
// differs. Positions are read from and written back to the chain-order
// global array; the caller rebuilds the global cell histogram afterwards.
//
// Shared memory per bead: position (16 B), cell-ordered copy (16 B), stage-1
// force (12 B), pair force / stage-1 position (12 B), slot and rank (2 + 2
// B); per cell one 32-bit count/start. About 2,900 beads fit a CTA.
#pragma once

#include "kernels.cuh"

namespace ccpgpu {

// Cell grid of one system inside the persistent kernel: a cube of cps^3
// cells of side 1 / inv_csl centred at the origin.
struct PGrid {
  int32_t cps;
  float inv_csl;
  int32_t n_cells;  // cps^3
  int32_t pad;
};

constexpr int PERSIST_THREADS = 512;

__host__ __device__ constexpr size_t persist_align(size_t x) { return (x + 15) & ~size_t(15); }

// Shared-memory bytes of a system of n beads and c cells.
__host__ __device__ constexpr size_t persist_smem_bytes(int n, int c) {
  return persist_align(16 * (size_t)n) * 2 + persist_align(12 * (size_t)n) * 2 +
         persist_align(2 * (size_t)n) * 2 + persist_align(4 * ((size_t)c + 1));
}

struct PersistSmem {
  float4 *r;       // chain order: current positions, flags in w
  float4 *sorted;  // cell order: x, y, z, (index << BF_BITS) | flags
  float3 *f1;      // chain order: stage-1 force
  float3 *fs;      // cell order: pair forces; after stage 1 the stage-1 positions
  uint16_t *slot;  // chain order: slot of the bead in `sorted`
  uint16_t *rank;  // chain order: rank of the bead in its cell (histogram)
  uint32_t *cell;  // cell counts, then exclusive starts; cell[n_cells] = n
};

__device__ __forceinline__ PersistSmem persist_carve(unsigned char *base, int n) {
  PersistSmem m;
  size_t o = 0;
  m.r = reinterpret_cast<float4 *>(base + o);
  o += persist_align(16 * (size_t)n);
  m.sorted = reinterpret_cast<float4 *>(base + o);
  o += persist_align(16 * (size_t)n);
  m.f1 = reinterpret_cast<float3 *>(base + o);
  o += persist_align(12 * (size_t)n);
  m.fs = reinterpret_cast<float3 *>(base + o);
  o += persist_align(12 * (size_t)n);
  m.slot = reinterpret_cast<uint16_t *>(base + o);
  o += persist_align(2 * (size_t)n);
  m.rank = reinterpret_cast<uint16_t *>(base + o);
  o += persist_align(2 * (size_t)n);
  m.cell = reinterpret_cast<uint32_t *>(base + o);
  return m;
}

__device__ __forceinline__ CellXYZ persist_cell_xyz(float4 p, const PGrid &g, bool &esc) {
  CellXYZ c;
  c.x = cell_coord(p.x, g.inv_csl, g.cps, esc);
  c.y = cell_coord(p.y, g.inv_csl, g.cps, esc);
  c.z = cell_coord(p.z, g.inv_csl, g.cps, esc);
  return c;
}

__device__ __forceinline__ int persist_cell(float4 p, const PGrid &g, int *err) {
  bool esc = false;
  CellXYZ c = persist_cell_xyz(p, g, esc);
  if (esc) set_err(err, ERR_ESCAPE);
  return (c.z * g.cps + c.y) * g.cps + c.x;
}

// Exclusive scan of cell[0 .. nc) in place, cell[nc] = the total. Each thread
// scans one contiguous chunk; the chunk sums are scanned across the block.
__device__ __forceinline__ void persist_scan(uint32_t *cell, int nc) {
  __shared__ uint32_t tot;
  const int per = (nc + PERSIST_THREADS - 1) / PERSIST_THREADS;
  const int b = min((int)threadIdx.x * per, nc), e = min(b + per, nc);
  uint32_t sum = 0;
  for (int c = b; c < e; ++c) sum += cell[c];
  uint32_t off = block_excl_scan<PERSIST_THREADS>(sum, &tot);
  for (int c = b; c < e; ++c) {
    uint32_t v = cell[c];
    cell[c] = off;
    off += v;
  }
  if (threadIdx.x == 0) cell[nc] = tot;
  __syncthreads();
}

// Half-shell pair pass over the cell-ordered copy (as k_pair_half): the bead
// in slot k visits the beads after it in its own row range and the forward
// rows of the (2 REACH + 1)^3 stencil; reactions go to fs by shared-memory
// atomics. fs must be zero on entry.
template <int MODE, int REACH>
__device__ __forceinline__ void persist_pairs(const PersistSmem &m, int n, const PGrid &g,
                                              const ForceField &ff) {
  const float rc_max = (MODE == MODE_ICG) ? ff.rc_icg : fmaxf(ff.rc_att, ff.rc_rep);
  const float rc2_max = rc_max * rc_max;
  const int cps = g.cps;
  for (int k = threadIdx.x; k < n; k += PERSIST_THREADS) {
    const float4 p = m.sorted[k];
    const uint32_t wi = wbits(p);
    bool esc = false;
    const CellXYZ c = persist_cell_xyz(p, g, esc);
    const int x0 = max(c.x - REACH, 0), x1 = min(c.x + REACH, cps - 1);
    float3 acc = make_float3(0.0f, 0.0f, 0.0f);
    auto range = [&](int b, int e) {
      for (int j = b; j < e; ++j) {
        const float4 q = m.sorted[j];
        const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
        const float d2 = dx * dx + dy * dy + dz * dz;
        if (d2 > rc2_max) continue;
        const uint32_t wj = wbits(q);
        const bool hh = (wi & wj & BF_HET) != 0u;
        if (MODE != MODE_ICG) {
          const float rc = hh ? ff.rc_att : ff.rc_rep;
          if (d2 > rc * rc) continue;
        }
        const int gi = (int)(wi >> BF_BITS), gj = (int)(wj >> BF_BITS);
        if ((unsigned)(gi - gj + 1) <= 2u) continue;
        const float cf = pair_coef<MODE>(dx, dy, dz, d2, hh, ff);
        const float fx = cf * dx, fy = cf * dy, fz = cf * dz;
        acc.x += fx;
        acc.y += fy;
        acc.z += fz;
        atomicAdd(&m.fs[j].x, -fx);
        atomicAdd(&m.fs[j].y, -fy);
        atomicAdd(&m.fs[j].z, -fz);
      }
    };
    range(k + 1, (int)m.cell[(c.z * cps + c.y) * cps + x1 + 1]);
    constexpr int NR = REACH + REACH * (2 * REACH + 1);
#pragma unroll 1
    for (int r = 0; r < NR; ++r) {
      int y, z;
      if (r < REACH) {
        y = c.y + 1 + r;
        z = c.z;
      } else {
        const int q = r - REACH;
        y = c.y - REACH + q % (2 * REACH + 1);
        z = c.z + 1 + q / (2 * REACH + 1);
      }
      if (y < 0 || y >= cps || z >= cps) continue;
      const int row = (z * cps + y) * cps;
      range((int)m.cell[row + x0], (int)m.cell[row + x1 + 1]);
    }
    atomicAdd(&m.fs[k].x, acc.x);
    atomicAdd(&m.fs[k].y, acc.y);
    atomicAdd(&m.fs[k].z, acc.z);
  }
}

// Forces other than the pair forces on bead i at position x (chain neighbours
// through X): bonded + bending, wall, lamina binding.
template <int MODE, class Load>
__device__ __forceinline__ float3 persist_local_force(Load X, int i, float4 x, int n,
                                                      const SysDesc &s, const ForceField &ff,
                                                      const float4 *__restrict__ lbs,
                                                      const uint32_t *__restrict__ lbs_start) {
  float3 F = bonded_force_at(X, i, x, n, ff);
  float3 vw;
  float gh, gl;
  if (wall_vector<MODE>(make_float3(x.x, x.y, x.z), s, vw, gh, gl)) {
    const float cw = wall_coef<MODE>(gh, gl, ff);
    F.x += cw * vw.x;
    F.y += cw * vw.y;
    F.z += cw * vw.z;
  }
  if (MODE == MODE_DST && (wbits(x) & BF_LAD) && s.n_lbs > 0) {
    const float3 fl = lbs_force(x, s, ff, lbs, lbs_start);
    F.x += fl.x;
    F.y += fl.y;
    F.z += fl.z;
  }
  return F;
}

template <int MODE>
__device__ __forceinline__ float3 persist_noise(int i, uint64_t st, const SysDesc &s,
                                                const ForceField &ff, int *err) {
  if (MODE != MODE_DST || !(ff.sd > 0.0f)) return make_float3(0.0f, 0.0f, 0.0f);
  const float3 z = bead_noise((uint32_t)i, st, s.seed_lo, s.seed_hi, err);
  return make_float3(ff.sd * z.x, ff.sd * z.y, ff.sd * z.z);
}

// nsteps Heun steps of system blockIdx.x; step0 is the step index of the
// first (the noise counter of the graph path's k_update).
template <int MODE, int REACH>
__global__ void __launch_bounds__(PERSIST_THREADS, 1)
    k_persist(const SysDesc *__restrict__ sys, const PGrid *__restrict__ grids, ForceField ff,
              float4 *__restrict__ pos, const float4 *__restrict__ lbs,
              const uint32_t *__restrict__ lbs_start, unsigned long long step0, int nsteps,
              int *__restrict__ err) {
  extern __shared__ __align__(16) unsigned char persist_shared[];
  const SysDesc &s = sys[blockIdx.x];
  const PGrid g = grids[blockIdx.x];
  const int n = s.n, nc = g.n_cells;
  const PersistSmem m = persist_carve(persist_shared, n);
  const int T = PERSIST_THREADS;
  const float h = 0.5f * ff.dt;

  for (int c = threadIdx.x; c <= nc; c += T) m.cell[c] = 0u;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += T) {
    const float4 x = pos[s.bead_off + i];
    m.r[i] = x;
    m.rank[i] = (uint16_t)atomicAdd(&m.cell[persist_cell(x, g, err)], 1u);
  }
  __syncthreads();

  for (int hs = 0; hs < nsteps; ++hs) {
    const uint64_t st = step0 + (uint64_t)hs;
    // ---- stage 1: forces at r
    persist_scan(m.cell, nc);
    for (int i = threadIdx.x; i < n; i += T) {
      const float4 x = m.r[i];
      const int k = (int)m.cell[persist_cell(x, g, err)] + m.rank[i];
      m.slot[i] = (uint16_t)k;
      m.sorted[k] = make_float4(x.x, x.y, x.z, __uint_as_float(((uint32_t)i << BF_BITS) |
                                                                (wbits(x) & 7u)));
      m.fs[k] = make_float3(0.0f, 0.0f, 0.0f);
    }
    __syncthreads();
    persist_pairs<MODE, REACH>(m, n, g, ff);
    __syncthreads();
    for (int c = threadIdx.x; c <= nc; c += T) m.cell[c] = 0u;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += T) {
      const float4 x = m.r[i];
      const int k = m.slot[i];
      float3 F = m.fs[k];
      const float3 fl = persist_local_force<MODE>([&](int j) { return m.r[j]; }, i, x, n, s, ff,
                                                  lbs, lbs_start);
      F.x += fl.x;
      F.y += fl.y;
      F.z += fl.z;
      const float3 rn = persist_noise<MODE>(i, st, s, ff, err);
      m.f1[i] = F;
      float3 D = make_float3(F.x * ff.dt, F.y * ff.dt, F.z * ff.dt);
      cap_step(D, MODE == MODE_ICG ? ff.icg_max_step : ff.max_step);
      const float4 e = make_float4(x.x + D.x + rn.x, x.y + D.y + rn.y, x.z + D.z + rn.z, x.w);
      m.fs[k] = make_float3(e.x, e.y, e.z);  // this slot's pair force is consumed
      if (!(isfinite(e.x) && isfinite(e.y) && isfinite(e.z))) set_err(err, ERR_NAN);
      m.rank[i] = (uint16_t)atomicAdd(&m.cell[persist_cell(e, g, err)], 1u);
    }
    __syncthreads();
    // ---- stage 2: forces at the stage-1 positions
    persist_scan(m.cell, nc);
    for (int i = threadIdx.x; i < n; i += T) {
      const float3 e3 = m.fs[m.slot[i]];
      const float4 e = make_float4(e3.x, e3.y, e3.z, m.r[i].w);
      const int k = (int)m.cell[persist_cell(e, g, err)] + m.rank[i];
      m.sorted[k] = make_float4(e.x, e.y, e.z, __uint_as_float(((uint32_t)i << BF_BITS) |
                                                                (wbits(e) & 7u)));
      m.rank[i] = (uint16_t)k;  // the new slot; slot[i] still names the stage-1 position
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += T) {
      m.slot[i] = m.rank[i];
      m.fs[i] = make_float3(0.0f, 0.0f, 0.0f);
    }
    __syncthreads();
    persist_pairs<MODE, REACH>(m, n, g, ff);
    __syncthreads();
    for (int c = threadIdx.x; c <= nc; c += T) m.cell[c] = 0u;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += T) {
      const int k = m.slot[i];
      const float4 e = m.sorted[k];
      float3 F = m.fs[k];
      const float3 fl = persist_local_force<MODE>([&](int j) { return m.sorted[m.slot[j]]; }, i, e,
                                                  n, s, ff, lbs, lbs_start);
      F.x += fl.x;
      F.y += fl.y;
      F.z += fl.z;
      const float3 rn = persist_noise<MODE>(i, st, s, ff, err);
      const float4 x = m.r[i];
      const float3 f1 = m.f1[i];
      float3 D = make_float3((f1.x + F.x) * h, (f1.y + F.y) * h, (f1.z + F.z) * h);
      cap_step(D, MODE == MODE_ICG ? ff.icg_max_step : ff.max_step);
      const float4 o = make_float4(x.x + D.x + rn.x, x.y + D.y + rn.y, x.z + D.z + rn.z, x.w);
      if (!(isfinite(o.x) && isfinite(o.y) && isfinite(o.z))) set_err(err, ERR_NAN);
      m.rank[i] = (uint16_t)atomicAdd(&m.cell[persist_cell(o, g, err)], 1u);
      m.r[i] = o;  // read only by this thread in this pass (stage-2 neighbours come from sorted)
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < n; i += T) pos[s.bead_off + i] = m.r[i];
}

}  // namespace ccpgpu
