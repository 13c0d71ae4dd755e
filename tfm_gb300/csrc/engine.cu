// Batched GB300 Brownian-dynamics engine and its C ABI (include/ccpgpu.h).
//
// Memory layout in HBM (all systems concatenated, chain order):
//   pos, er          float4 per bead: x, y, z, flags (BF_*) in w
//   fbuf             float4 per bead: stage-1 force (f of chrsim.cu:387)
//   rnb              float4 per bead: the step's noise, drawn by stage 1 and
//                    reused by stage 2 (one rn per step, chrsim.cu:387, :415)
//   sorted           float4 per bead in cell order: x, y, z, (index << 3 | flags)
//   fs               float4 per bead in cell order: pair force
//   rank             uint32 per bead: rank of the bead inside its cell
//   counts           uint8 per cell: histogram (four cells per 32-bit word)
//   start            uint32 per cell (+1): exclusive prefix
// Cells of system s occupy [cell_off, cell_off + cps^3); because every system
// lives in its own cells, the counting sort keeps each system's beads inside
// its own slot range [bead_off, bead_off + n).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/ccpgpu.h"
#include "analysis.h"
#include "host.h"
#include "kernels.cuh"
#include "persist.cuh"

namespace ccpgpu {

#define CK(x)                                                                      \
  do {                                                                             \
    cudaError_t e_ = (x);                                                          \
    if (e_ != cudaSuccess) throw Error(ST_CUDA, std::string("cuda: ") + cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  void alloc(size_t n_) {
    release();
    n = n_;
    if (n) CK(cudaMalloc(&p, n * sizeof(T)));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  ~DevBuf() { release(); }
};

constexpr int TILE = 128;
constexpr int SMALL_BATCH = 16384;  // beads: below, tiles of 64 and 8 lanes per bead
constexpr int MAX_CPS = 1024;  // cells per side of one system's grid
constexpr uint32_t MAX_BATCH_BEADS = (1u << (32u - BF_BITS)) - 1u;
constexpr int64_t MAX_BATCH_CELLS = (int64_t)INT32_MAX - 4 * (int64_t)SCAN_CHUNK;

// Host copy of a large position array split over a few threads: one thread
// copies well below the host's memory bandwidth, and the end-to-end path
// copies the positions in and out every step.
static void host_copy(void *dst, const void *src, size_t bytes) {
  const size_t min_chunk = size_t(4) << 20;
  unsigned nt = std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
  nt = (unsigned)std::min<size_t>(nt, std::max<size_t>(1, bytes / min_chunk));
  if (nt <= 1) {
    std::memcpy(dst, src, bytes);
    return;
  }
  std::vector<std::thread> th;
  const size_t chunk = (bytes + nt - 1) / nt;
  for (unsigned k = 0; k < nt; ++k) {
    size_t b = k * chunk, e = std::min(bytes, b + chunk);
    if (b >= e) break;
    th.emplace_back([=] {
      std::memcpy(static_cast<char *>(dst) + b, static_cast<const char *>(src) + b, e - b);
    });
  }
  for (auto &t : th) t.join();
}

// Page-locked host storage, so that copies to and from the device run as DMA
// without a staging copy.
template <class T>
struct PinnedAlloc {
  using value_type = T;
  PinnedAlloc() = default;
  template <class U>
  PinnedAlloc(const PinnedAlloc<U> &) {}
  T *allocate(size_t n) {
    void *p = nullptr;
    if (cudaMallocHost(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess)
      throw std::bad_alloc();
    return static_cast<T *>(p);
  }
  void deallocate(T *p, size_t) { cudaFreeHost(p); }
  template <class U>
  bool operator==(const PinnedAlloc<U> &) const { return true; }
  template <class U>
  bool operator!=(const PinnedAlloc<U> &) const { return false; }
};
using PinnedFloats = std::vector<float, PinnedAlloc<float>>;

struct Engine {
  Params par;
  ForceField ff{};
  std::vector<SystemSpec> specs;
  std::vector<SysDesc> hsys;
  std::vector<Geometry> geo;
  std::vector<Tile> htiles;   // bead tiles (chain order / cell order)
  std::vector<Tile> hctiles;  // cell tiles: PAIR_WARPS cells of one x-row
  int nb = 0, nc = 0, nl = 0, nch = 0;
  int nblk = 0;        // scan CTAs
  int tile = TILE;     // beads per CTA of the per-bead kernels (64, 128 or 256)
  float need_cut = 0;  // largest interaction / contact cutoff: cell side >= need_cut / reach
  int64_t map_total = 0;
  int ps_total = 0;

  // host state
  PinnedFloats hxyz;           // chain-order positions (pinned)
  std::vector<int32_t> hpt;    // ccp type codes
  std::vector<float> hlbs;     // LBS positions, per system in placement order
  std::vector<uint32_t> hflags;
  std::vector<int32_t> chain_of, chain_first, chain_len, chain_ps_off, chain_smax, chain_sys;
  std::vector<uint32_t> i_f;
  std::vector<float> t;
  uint64_t step = 0;
  uint64_t dev_next = ~0ull;  // step the device counter will produce next
  int frames_observed = 0;
  bool positions_valid = false;

  // device state
  DevBuf<SysDesc> d_sys;
  DevBuf<Tile> d_tiles, d_ctiles;
  DevBuf<float4> pos, er, fbuf, rnb, fs, sorted, lbs_sorted, fout;
  DevBuf<uint32_t> rank, counts, start, bsum, lbs_start;
  DevBuf<int32_t> d_chain_of, d_chain_first, d_chain_len, d_chain_ps_off, d_chain_smax;
  DevBuf<int32_t> map, ps;
  DevBuf<double> obs, ds;
  // ccp-analyze's outputs (analysis.h): per-frame sums of the observables and
  // the nematic order / nucleus fraction sums of the frame being analysed
  Analysis ana;
  DevBuf<double> fobs, fextra;
  DevBuf<unsigned long long> ovl, d_step;
  DevBuf<int> d_err;
  DevBuf<float> xyz_stage;
  DevBuf<float> fstage[2];  // packed frames of run_simulation, alternating
  float *pinned[2] = {nullptr, nullptr};
  float4 *pin_up = nullptr;  // pinned staging of position uploads
  bool lbs_uploaded = false;
  bool flags_current = false;  // pos.w holds the flags of the current types
  cudaStream_t stream = nullptr;
  cudaStream_t cstream = nullptr;  // device-to-host frame copies
  cudaEvent_t ev[2] = {nullptr, nullptr};       // frame copy done (cstream)
  cudaEvent_t ev_pack[2] = {nullptr, nullptr};  // frame packed (stream)
  std::map<std::tuple<int, int, int>, cudaGraphExec_t> graphs;
  std::map<std::tuple<int, int, int>, uint64_t> graph_kernels;  // kernel nodes per graph
  uint64_t kcount = 0;  // engine kernels launched (graph nodes included)
  // persistent per-system path (persist.cuh): 0 when the batch does not use it
  int persist_reach = 0;
  size_t persist_bytes = 0;
  DevBuf<PGrid> d_pgrid;

  ~Engine() {
    for (auto &g : graphs) cudaGraphExecDestroy(g.second);
    for (int k = 0; k < 2; ++k) {
      if (pinned[k]) cudaFreeHost(pinned[k]);
      if (k == 0 && pin_up) cudaFreeHost(pin_up);
      if (ev[k]) cudaEventDestroy(ev[k]);
      if (ev_pack[k]) cudaEventDestroy(ev_pack[k]);
    }
    if (cstream) cudaStreamDestroy(cstream);
    if (stream) cudaStreamDestroy(stream);
  }

  // -------------------------------------------------------------- setup
  void build(const Params &p, std::vector<SystemSpec> sp) {
    par = p;
    ff = p.ff;
    specs = std::move(sp);
    int ns = (int)specs.size();
    int64_t beads = 0;
    for (const auto &q : specs) beads += q.n;
    check_totals(beads, 0);
    hsys.resize(ns);
    geo.resize(ns);
    i_f.assign(ns, 0);
    t.assign(ns, 0.0f);
    nb = nc = nl = nch = 0;
    map_total = 0;
    ps_total = 0;
    chain_of.clear();
    chain_first.clear();
    chain_len.clear();
    chain_ps_off.clear();
    chain_smax.clear();
    chain_sys.clear();
    for (int s = 0; s < ns; ++s) {
      SystemSpec &q = specs[s];
      Geometry g = make_geometry(q.R_n, q.R_o, q.R_b);
      geo[s] = g;
      SysDesc d{};
      d.bead_off = nb;
      d.n = q.n;
      d.csl = p.cell_side;
      d.inv_csl = 1.0f / p.cell_side;
      d.cps = grid_side(g.d_m, p.cell_side);
      check_totals(beads, (int64_t)nc + cells_of(d.cps));
      d.cell_off = nc;
      d.cls_cells = typed() ? d.cps * d.cps * d.cps : 0;
      d.R_n = g.R_n;
      d.R_o = g.R_o;
      d.R_b = g.R_b;
      d.noc = g.noc;
      d.boc = g.boc;
      d.nod = g.nod;
      d.bod = g.bod;
      d.lbs_off = nl;
      d.n_lbs = q.n_lbs;
      d.lbs_rmin = 1e30f;  // set from the sites by upload_lbs
      d.lbs_rmax = -1e30f;
      d.seed_lo = (uint32_t)q.seed;
      d.seed_hi = (uint32_t)(q.seed >> 32);
      d.chain_off = nch;
      d.sys_index = s;
      // chains
      std::vector<int> heads = q.chain_first;
      if (heads.empty()) {
        int L = q.n / q.n_chains;
        for (int c = 0; c < q.n_chains; ++c) heads.push_back(c * L);
      }
      d.n_chains = (int)heads.size();
      for (int c = 0; c < d.n_chains; ++c) {
        int b = heads[c], e = (c + 1 < d.n_chains) ? heads[c + 1] : q.n;
        chain_first.push_back(nb + b);
        chain_len.push_back(e - b);
        chain_smax.push_back((e - b) / 2);
        chain_ps_off.push_back(ps_total);
        chain_sys.push_back(s);
        ps_total += (e - b) / 2 + 1;
        for (int i = b; i < e; ++i) chain_of.push_back(nch + c);
      }
      nch += d.n_chains;
      // contact map binning (chrana.cu:187-189 for the ccp pixels)
      bool diploid = (p.preset == PRESET_CCP && (uint32_t)q.n == CCP_N_DEF && d.n_chains == 12);
      d.n_copies = diploid ? 2 : 1;
      d.copy_len = q.n / d.n_copies;
      if (q.contact_bins > 0) {
        d.nbins = std::min(q.contact_bins, d.copy_len);
        d.map_len = d.copy_len;
      } else {
        d.nbins = d.copy_len / CCP_PX_SZ;
        d.map_len = d.nbins * CCP_PX_SZ;
      }
      if (d.nbins < 1) {
        d.nbins = 1;
        d.map_len = d.copy_len;
      }
      d.map_off = map_total;
      map_total += (int64_t)d.nbins * (d.nbins + 1) / 2;
      hsys[s] = d;
      nb += q.n;
      nc += (int)cells_of(d.cps);
      nl += q.n_lbs;
    }
    need_cut = std::max({ff.rc_att, ff.rc_rep, ff.rc_icg, p.contact_cutoff, ff.mis});
    for (auto &d : hsys) d.reach = (d.csl >= need_cut) ? 1 : 2;
    // batches too small to fill the GPU: tiles of 64 beads, eight lanes per
    // bead in the pair pass (pair_lanes); measured on single ccp systems of
    // 1024-8192 beads 8-12 % faster per Heun step than tiles of 128 with four
    tile = (nb < SMALL_BATCH) ? 64 : TILE;
    build_tiles();
    nblk = (nc + 1 + SCAN_CHUNK - 1) / SCAN_CHUNK;

    hxyz.assign((size_t)3 * nb, 0.0f);
    hpt.assign(nb, 1);
    hlbs.assign((size_t)3 * nl, 0.0f);
    hflags.assign(nb, 0);

    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&cstream, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) {
      CK(cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&ev_pack[k], cudaEventDisableTiming));
    }
    d_sys.alloc(ns);
    d_tiles.alloc(htiles.size());
    d_ctiles.alloc(hctiles.size());
    pos.alloc(nb + 1);
    er.alloc(nb + 1);
    fbuf.alloc(nb + 1);
    rnb.alloc(nb + 1);
    fs.alloc(nb + 1);
    sorted.alloc(nb + 1);
    fout.alloc(nb + 1);
    rank.alloc(nb + 1);
    size_t cpad = (size_t)nblk * SCAN_CHUNK;
    counts.alloc(cpad / 4);  // byte counts
    start.alloc(cpad + 4);
    bsum.alloc(nblk + 1);
    lbs_sorted.alloc(std::max(nl, 1));
    lbs_start.alloc(nc + 1);
    d_chain_of.alloc(nb);
    d_chain_first.alloc(nch);
    d_chain_len.alloc(nch);
    d_chain_ps_off.alloc(nch);
    d_chain_smax.alloc(nch);
    map.alloc(std::max<int64_t>(map_total, 1));
    ps.alloc(std::max(ps_total, 1));
    ds.alloc(std::max(ps_total, 1));
    obs.alloc((size_t)ns * OBS_STRIDE);
    ovl.alloc(ns);
    d_step.alloc(1);
    d_err.alloc(ERR_COUNT);
    xyz_stage.alloc((size_t)3 * nb);
    for (int k = 0; k < 2; ++k) {
      fstage[k].alloc((size_t)3 * nb);
      CK(cudaMallocHost(&pinned[k], sizeof(float) * 3 * std::max(nb, 1)));
    }
    CK(cudaMallocHost(&pin_up, sizeof(float4) * (nb + 1)));

    CK(cudaMemcpyAsync(d_sys.p, hsys.data(), sizeof(SysDesc) * ns, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_tiles.p, htiles.data(), sizeof(Tile) * htiles.size(),
                       cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_ctiles.p, hctiles.data(), sizeof(Tile) * hctiles.size(),
                       cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_chain_of.p, chain_of.data(), 4 * nb, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_chain_first.p, chain_first.data(), 4 * nch, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_chain_len.p, chain_len.data(), 4 * nch, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_chain_ps_off.p, chain_ps_off.data(), 4 * nch, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_chain_smax.p, chain_smax.data(), 4 * nch, cudaMemcpyHostToDevice, stream));
    CK(cudaMemsetAsync(counts.p, 0, cpad, stream));
    CK(cudaMemsetAsync(start.p, 0, sizeof(uint32_t) * (cpad + 4), stream));
    CK(cudaMemsetAsync(d_err.p, 0, sizeof(int) * ERR_COUNT, stream));
    CK(cudaMemsetAsync(pos.p, 0, sizeof(float4) * (nb + 1), stream));
    CK(cudaMemsetAsync(er.p, 0, sizeof(float4) * (nb + 1), stream));
    CK(cudaMemsetAsync(fbuf.p, 0, sizeof(float4) * (nb + 1), stream));
    CK(cudaMemsetAsync(rnb.p, 0, sizeof(float4) * (nb + 1), stream));
    CK(cudaMemsetAsync(fs.p, 0, sizeof(float4) * (nb + 1), stream));
    CK(cudaMemsetAsync(sorted.p, 0, sizeof(float4) * (nb + 1), stream));
    CK(cudaMemsetAsync(lbs_start.p, 0, sizeof(uint32_t) * (nc + 1), stream));
    reset_observables();
    setup_persist();
    CK(cudaStreamSynchronize(stream));
  }

  // Shared-memory cell grids of the persistent path: cells of the largest
  // pair cutoff over 2 (5x5x5 stencil) when every system then fits one CTA's
  // shared memory, else cells of the cutoff (3x3x3), else the path is off.
  void setup_persist() {
    persist_reach = 0;
    persist_bytes = 0;
    if (!par.persistent) return;
    int dev = 0, optin = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const size_t limit = (size_t)optin - 1024;  // the scan's static shared words
    // a margin above the cutoff keeps pairs at it within the stencil despite
    // the rounding of the cell coordinates
    const float rc = std::max({ff.rc_att, ff.rc_rep, ff.rc_icg}) * 1.0001f;
    const int ns = (int)hsys.size();
    for (int reach = 2; reach >= 1; --reach) {
      std::vector<PGrid> g(ns);
      size_t bytes = 0;
      bool ok = true;
      for (int s = 0; s < ns && ok; ++s) {
        const float csl = rc / (float)reach;
        const float half = std::ceil(geo[s].d_m / csl);
        if (!(half <= 64.0f) || hsys[s].n > 65535) {
          ok = false;
          break;
        }
        const int cps = std::max(2, 2 * (int)half);
        g[s] = PGrid{cps, 1.0f / csl, cps * cps * cps, 0};
        bytes = std::max(bytes, persist_smem_bytes(hsys[s].n, g[s].n_cells));
        ok = bytes <= limit;
      }
      if (!ok) continue;
      d_pgrid.alloc(ns);
      CK(cudaMemcpyAsync(d_pgrid.p, g.data(), sizeof(PGrid) * ns, cudaMemcpyHostToDevice, stream));
      if (reach == 2) {
        CK(cudaFuncSetAttribute(k_persist<MODE_DST, 2>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
        CK(cudaFuncSetAttribute(k_persist<MODE_ICG, 2>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
      } else {
        CK(cudaFuncSetAttribute(k_persist<MODE_DST, 1>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
        CK(cudaFuncSetAttribute(k_persist<MODE_ICG, 1>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
      }
      persist_reach = reach;
      persist_bytes = bytes;
      return;
    }
  }

  // g Heun steps of every system in one launch (one CTA per system).
  void launch_persist(int mode, int g) {
    const unsigned ns = (unsigned)hsys.size();
    const unsigned long long s0 = (unsigned long long)step;
#define CCPGPU_PERSIST(M, R)                                                              \
  k_persist<M, R><<<ns, PERSIST_THREADS, persist_bytes, stream>>>(                        \
      d_sys.p, d_pgrid.p, ff, pos.p, lbs_sorted.p, lbs_start.p, s0, g, d_err.p)
    if (mode == MODE_DST && persist_reach == 2)
      CCPGPU_PERSIST(MODE_DST, 2);
    else if (mode == MODE_DST)
      CCPGPU_PERSIST(MODE_DST, 1);
    else if (persist_reach == 2)
      CCPGPU_PERSIST(MODE_ICG, 2);
    else
      CCPGPU_PERSIST(MODE_ICG, 1);
#undef CCPGPU_PERSIST
    CK(cudaGetLastError());
    kcount += 1;
  }

  void build_tiles() {
    htiles.clear();
    for (int s = 0; s < (int)hsys.size(); ++s)
      for (int b = 0; b < hsys[s].n; b += tile) htiles.push_back(Tile{s, hsys[s].bead_off + b});
    hctiles.clear();
    for (int s = 0; s < (int)hsys.size(); ++s) {
      const int cps = hsys[s].cps;
      for (int row = 0; row < cps * cps; ++row)
        for (int x = 0; x < cps; x += PAIR_WARPS)
          hctiles.push_back(Tile{s, hsys[s].cell_off + row * cps + x});
    }
  }

  // -------------------------------------------------------------- uploads
  void set_chain_flags() {
    for (int i = 0; i < nb; ++i) hflags[i] = type_to_flags(hpt[i], par.preset);
    for (int c = 0; c < nch; ++c) hflags[chain_first[c]] |= BF_START;
  }

  // Uploads positions + flags (through pinned staging) and rebuilds the cell
  // histogram of pos.
  // count = false: the positions are placeholders about to be overwritten
  // (they would all fall into one cell), so no histogram is built.
  void upload_positions(bool count = true) {
    set_chain_flags();
    float4 *v = pin_up;
    for (int i = 0; i < nb; ++i) {
      uint32_t w = hflags[i];
      float wf;
      std::memcpy(&wf, &w, 4);
      v[i] = make_float4(hxyz[3 * i], hxyz[3 * i + 1], hxyz[3 * i + 2], wf);
    }
    uint32_t ws = BF_START;
    float wsf;
    std::memcpy(&wsf, &ws, 4);
    v[nb] = make_float4(0, 0, 0, wsf);
    CK(cudaMemcpyAsync(pos.p, v, sizeof(float4) * (nb + 1), cudaMemcpyHostToDevice, stream));
    if (count) recount();
    CK(cudaStreamSynchronize(stream));
    positions_valid = true;
    flags_current = true;
  }

  // New positions only (hxyz), the flags already on the device: one DMA of
  // the xyz triples and a kernel that writes them under the flags.
  void upload_xyz() {
    if (!flags_current || !positions_valid) {
      upload_positions();
      return;
    }
    CK(cudaMemcpyAsync(xyz_stage.p, hxyz.data(), sizeof(float) * 3 * nb, cudaMemcpyHostToDevice,
                       stream));
    k_unpack_xyz<<<(nb + 255) / 256, 256, 0, stream>>>(xyz_stage.p, pos.p, nb);
    CK(cudaGetLastError());
    recount();
    CK(cudaStreamSynchronize(stream));
  }

  void recount() {
    CK(cudaMemsetAsync(counts.p, 0, (size_t)nblk * SCAN_CHUNK, stream));
    k_count<<<(unsigned)htiles.size(), tile, 0, stream>>>(d_tiles.p, d_sys.p, pos.p, counts.p,
                                                           rank.p, d_err.p);
    CK(cudaGetLastError());
    kcount += 1;
  }

  // LBS of every system sorted by cell (static during a run).
  void upload_lbs() {
    std::vector<uint32_t> cnt(nc + 1, 0);
    std::vector<int> cell_of_l(nl);
    for (size_t s = 0; s < hsys.size(); ++s) {
      SysDesc &d = hsys[s];
      d.lbs_rmin = 1e30f;
      d.lbs_rmax = -1e30f;
      for (int k = 0; k < d.n_lbs; ++k) {
        int l = d.lbs_off + k;
        float r = std::sqrt(hlbs[3 * l] * hlbs[3 * l] + hlbs[3 * l + 1] * hlbs[3 * l + 1] +
                            hlbs[3 * l + 2] * hlbs[3 * l + 2]);
        d.lbs_rmin = std::min(d.lbs_rmin, r * 0.9999f - 1e-4f);
        d.lbs_rmax = std::max(d.lbs_rmax, r * 1.0001f + 1e-4f);
        int c[3];
        for (int a = 0; a < 3; ++a) {
          float v = hlbs[3 * l + a];
          float f = std::floor(v * d.inv_csl) + (float)(d.cps >> 1);
          int ci = (f >= 0.0f) ? ((f >= (float)d.cps) ? d.cps - 1 : (int)f) : 0;
          c[a] = ci;
        }
        int cl = d.cell_off + (c[2] * d.cps + c[1]) * d.cps + c[0];
        cell_of_l[l] = cl;
        cnt[cl]++;
      }
    }
    std::vector<uint32_t> st(nc + 1, 0);
    uint32_t acc = 0;
    for (int c = 0; c < nc; ++c) {
      st[c] = acc;
      acc += cnt[c];
    }
    st[nc] = acc;
    std::vector<float4> srt(std::max(nl, 1));
    std::vector<uint32_t> fill(st.begin(), st.end());
    for (int l = 0; l < nl; ++l) {
      uint32_t slot = fill[cell_of_l[l]]++;
      srt[slot] = make_float4(hlbs[3 * l], hlbs[3 * l + 1], hlbs[3 * l + 2], 0.0f);
    }
    CK(cudaMemcpyAsync(lbs_sorted.p, srt.data(), sizeof(float4) * std::max(nl, 1),
                       cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(lbs_start.p, st.data(), sizeof(uint32_t) * (nc + 1), cudaMemcpyHostToDevice,
                       stream));
    CK(cudaMemcpyAsync(d_sys.p, hsys.data(), sizeof(SysDesc) * hsys.size(), cudaMemcpyHostToDevice,
                       stream));
    CK(cudaStreamSynchronize(stream));
    lbs_uploaded = true;
  }

  void download_positions() {
    k_pack_xyz<<<(nb + 255) / 256, 256, 0, stream>>>(pos.p, xyz_stage.p, nb);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(hxyz.data(), xyz_stage.p, sizeof(float) * 3 * nb, cudaMemcpyDeviceToHost,
                       stream));
    CK(cudaStreamSynchronize(stream));
  }

  // -------------------------------------------------------------- launches
  void launch_scan(bool bump) {
    k_scan_reduce<<<nblk, SCAN_THREADS, 0, stream>>>(counts.p, bsum.p);
    k_scan_top<<<1, SCAN_TOP_THREADS, 0, stream>>>(bsum.p, nblk, d_step.p, bump ? 1 : 0);
    k_scan_apply<<<nblk, SCAN_THREADS, 0, stream>>>(counts.p, bsum.p, start.p, nc, nblk);
    kcount += 3;
  }

  void launch_scatter(const float4 *src) {
    k_scatter<<<(unsigned)htiles.size(), tile, 0, stream>>>(
        d_tiles.p, d_sys.p, src, rank.p, start.p, sorted.p,
        par.pair_kernel >= 2 ? fs.p : nullptr, counts.p, d_err.p);
    kcount += 1;
  }

  // Typed layout (pair_kernel 4): A beads and the others sorted into separate
  // cell grids of each system.
  bool typed() const { return par.pair_kernel == 4; }

  // Cells per side of a system's grid: the cube of side 2 d_m (d_m = the
  // largest distance of a bead from the centre) in cells of side csl.
  static int grid_side(float d_m, float csl) {
    float half = std::ceil(d_m / csl);
    if (!(half <= (float)(MAX_CPS / 2)))
      throw Error(ST_ARG, "nucleus too large for the cell side (more than " +
                              std::to_string(MAX_CPS) + " cells per side)");
    return std::max(2, 2 * (int)half);
  }

  // Cells of one system: one grid, or two in the typed layout.
  int64_t cells_of(int cps) const { return (typed() ? 2 : 1) * (int64_t)cps * cps * cps; }

  // The sorted words carry a bead's batch index in 32 - BF_BITS bits, and
  // cells are addressed with 32-bit ints (plus the scan's padding).
  static void check_totals(int64_t beads, int64_t cells) {
    if (beads > (int64_t)MAX_BATCH_BEADS)
      throw Error(ST_ARG, "batch holds more than " + std::to_string(MAX_BATCH_BEADS) + " beads");
    if (cells > MAX_BATCH_CELLS)
      throw Error(ST_ARG, "batch needs more than " + std::to_string(MAX_BATCH_CELLS) +
                              " cells; use a larger cell_side or fewer systems");
  }

  // Stencil reaches of the typed pair kernel for MODE when every system has
  // the same (A-A reach * 4 + other reach), else 0.
  template <int MODE>
  int typed_reaches() const {
    const float rhh = (MODE == MODE_ICG) ? ff.rc_icg : ff.rc_att;
    const float rx = (MODE == MODE_ICG) ? ff.rc_icg : ff.rc_rep;
    int key = -1;
    for (const auto &d : hsys) {
      int k = (d.csl >= rhh ? 1 : 2) * 4 + (d.csl >= rx ? 1 : 2);
      if (key >= 0 && k != key) return 0;
      key = k;
    }
    return key < 0 ? 0 : key;
  }

  // Lanes per bead of the half-shell pair kernels: the pair_lanes parameter,
  // or by the batch's bead count (more lanes for batches too small to fill
  // the GPU with one thread per bead).
  int pair_lanes() const {
    if (par.pair_lanes > 0) return par.pair_lanes;
    return nb < SMALL_BATCH ? 8 : (nb < 65536 ? 4 : (nb < 262144 ? 2 : 1));
  }

  template <int MODE, int RHH, int RX>
  void launch_typed(unsigned nt) {
    const int L = (tile * pair_lanes() <= 512) ? pair_lanes() : 1;
    if (L == 8)
      k_pair_typed_lanes<MODE, RHH, RX, 8><<<nt, (unsigned)(tile * 8), 0, stream>>>(
          d_tiles.p, d_sys.p, ff, sorted.p, start.p, fs.p);
    else if (L == 4)
      k_pair_typed_lanes<MODE, RHH, RX, 4><<<nt, (unsigned)(tile * 4), 0, stream>>>(
          d_tiles.p, d_sys.p, ff, sorted.p, start.p, fs.p);
    else if (L == 2)
      k_pair_typed_lanes<MODE, RHH, RX, 2><<<nt, (unsigned)(tile * 2), 0, stream>>>(
          d_tiles.p, d_sys.p, ff, sorted.p, start.p, fs.p);
    else
      k_pair_typed<MODE, RHH, RX><<<nt, tile, 0, stream>>>(d_tiles.p, d_sys.p, ff, sorted.p,
                                                           start.p, fs.p);
  }

  template <int MODE>
  void launch_pair() {
    const unsigned nt = (unsigned)htiles.size();
    if (par.pair_kernel == 4) {
      switch (typed_reaches<MODE>()) {
        case 2 * 4 + 1:
          launch_typed<MODE, 2, 1>(nt);
          break;
        case 1 * 4 + 1:
          launch_typed<MODE, 1, 1>(nt);
          break;
        case 2 * 4 + 2:
          launch_typed<MODE, 2, 2>(nt);
          break;
        default:  // systems gridded differently: each system's own reaches
          k_pair_typed<MODE, 0, 0><<<nt, tile, 0, stream>>>(d_tiles.p, d_sys.p, ff, sorted.p,
                                                             start.p, fs.p);
      }
    } else if (par.pair_kernel == 0)
      k_pair<MODE><<<(unsigned)htiles.size(), tile, 0, stream>>>(d_tiles.p, d_sys.p, ff, sorted.p,
                                                                  start.p, fs.p);
    else if (par.pair_kernel == 3 && par.reach == 2)
      k_pair_flat<MODE, 2><<<(unsigned)htiles.size(), tile, 0, stream>>>(d_tiles.p, d_sys.p, ff,
                                                                          sorted.p, start.p, fs.p);
    else if (par.pair_kernel == 3)
      k_pair_flat<MODE><<<(unsigned)htiles.size(), tile, 0, stream>>>(d_tiles.p, d_sys.p, ff,
                                                                       sorted.p, start.p, fs.p);
    else if (par.pair_kernel == 2 && pair_lanes() > 1 && uniform_reach() > 0 &&
             tile * pair_lanes() <= 512) {
      const unsigned bs = (unsigned)(tile * pair_lanes());
      const int r = uniform_reach();
      if (pair_lanes() == 2 && r == 2)
        k_pair_half_lanes<MODE, 2, 2><<<nt, bs, 0, stream>>>(d_tiles.p, d_sys.p, ff, sorted.p,
                                                             start.p, fs.p);
      else if (pair_lanes() == 2)
        k_pair_half_lanes<MODE, 1, 2><<<nt, bs, 0, stream>>>(d_tiles.p, d_sys.p, ff, sorted.p,
                                                             start.p, fs.p);
      else if (pair_lanes() == 8 && r == 2)
        k_pair_half_lanes<MODE, 2, 8><<<nt, bs, 0, stream>>>(d_tiles.p, d_sys.p, ff, sorted.p,
                                                             start.p, fs.p);
      else if (pair_lanes() == 8)
        k_pair_half_lanes<MODE, 1, 8><<<nt, bs, 0, stream>>>(d_tiles.p, d_sys.p, ff, sorted.p,
                                                             start.p, fs.p);
      else if (r == 2)
        k_pair_half_lanes<MODE, 2, 4><<<nt, bs, 0, stream>>>(d_tiles.p, d_sys.p, ff, sorted.p,
                                                             start.p, fs.p);
      else
        k_pair_half_lanes<MODE, 1, 4><<<nt, bs, 0, stream>>>(d_tiles.p, d_sys.p, ff, sorted.p,
                                                             start.p, fs.p);
    } else if (par.pair_kernel == 2 && uniform_reach() == 2)
      k_pair_half<MODE, 2><<<(unsigned)htiles.size(), tile, 0, stream>>>(d_tiles.p, d_sys.p, ff,
                                                                          sorted.p, start.p, fs.p);
    else if (par.pair_kernel == 2 && uniform_reach() == 1)
      k_pair_half<MODE, 1><<<(unsigned)htiles.size(), tile, 0, stream>>>(d_tiles.p, d_sys.p, ff,
                                                                          sorted.p, start.p, fs.p);
    else if (par.pair_kernel == 2)  // mixed: each system's own stencil reach
      k_pair_half<MODE, 0><<<(unsigned)htiles.size(), tile, 0, stream>>>(d_tiles.p, d_sys.p, ff,
                                                                          sorted.p, start.p, fs.p);
    else
      k_pair_cells<MODE><<<(unsigned)hctiles.size(), PAIR_WARPS * 32, 0, stream>>>(
          d_ctiles.p, d_sys.p, ff, sorted.p, start.p, fs.p);
    kcount += 1;
  }

  template <int STAGE, int MODE>
  void launch_update() {
    k_update<STAGE, MODE><<<(unsigned)htiles.size(), tile, 0, stream>>>(
        d_tiles.p, d_sys.p, ff, pos.p, er.p, fbuf.p, rnb.p, fs.p, rank.p, counts.p, lbs_sorted.p,
        lbs_start.p, d_step.p, d_err.p);
    kcount += 1;
  }

  ContactArgs contact_args(bool do_map, bool do_ps, bool do_ovl) {
    ContactArgs a;
    a.cut = par.contact_cutoff;
    a.mis = ff.mis;
    a.do_map = do_map;
    a.do_ps = do_ps;
    a.do_overlap = do_ovl;
    a.map = map.p;
    a.ps = ps.p;
    a.chain_of = d_chain_of.p;
    a.chain_first = d_chain_first.p;
    a.chain_ps_off = d_chain_ps_off.p;
    a.chain_smax = d_chain_smax.p;
    a.overlaps = ovl.p;
    return a;
  }

  // Observables on the cell-ordered copy of pos (must be current).
  // 1 or 2 when every system uses that stencil reach, 0 when they differ
  int uniform_reach() const {
    int r = hsys.empty() ? 1 : hsys[0].reach;
    for (const auto &d : hsys)
      if (d.reach != r) return 0;
    return r;
  }

  void launch_contacts_args(const ContactArgs &a) {
    const int r = uniform_reach();
    if (r == 1)
      k_contacts_half<1><<<(unsigned)htiles.size(), tile, 0, stream>>>(d_tiles.p, d_sys.p, sorted.p,
                                                                    start.p, a);
    else if (r == 2)
      k_contacts_half<2><<<(unsigned)htiles.size(), tile, 0, stream>>>(d_tiles.p, d_sys.p, sorted.p,
                                                                    start.p, a);
    else
      k_contacts_half<0><<<(unsigned)htiles.size(), tile, 0, stream>>>(d_tiles.p, d_sys.p, sorted.p,
                                                                    start.p, a);
    kcount += 1;
  }

  void launch_contacts() { launch_contacts_args(contact_args(true, true, false)); }

  void launch_observe() {
    k_observe<<<(unsigned)htiles.size(), tile, 0, stream>>>(d_tiles.p, d_sys.p, pos.p,
                                                             CCP_RCO / 2.0f, obs.p);
    kcount += 1;
  }

  void launch_observe_sorted(bool with_sdist) {
    launch_contacts();
    launch_observe();
    if (with_sdist) {
      int smax = 0, lmax = 0;
      for (int c = 0; c < nch; ++c) {
        smax = std::max(smax, chain_smax[c]);
        lmax = std::max(lmax, chain_len[c]);
      }
      if (smax > 0) {
        for (int c = 0; c < nch; ++c) {
          dim3 grid((chain_smax[c] + 127) / 128, (chain_len[c] + SDIST_PCHUNK - 1) / SDIST_PCHUNK);
          if (chain_smax[c] == 0) continue;
          k_sdist<<<grid, 128, 0, stream>>>(pos.p, d_chain_first.p, d_chain_len.p,
                                            d_chain_ps_off.p, d_chain_smax.p, c, ds.p);
          kcount += 1;
        }
      }
    }
  }

  template <int MODE>
  void launch_step(bool observe) {
    launch_scan(true);
    launch_scatter(pos.p);
    if (observe) launch_observe_sorted(false);
    launch_pair<MODE>();
    launch_update<1, MODE>();
    launch_scan(false);
    launch_scatter(er.p);
    launch_pair<MODE>();
    launch_update<2, MODE>();
  }

  // Graph of n steps; when obs is set the state at the first step is observed.
  cudaGraphExec_t graph_for(int mode, int n, bool obs) {
    auto key = std::make_tuple(mode, n, obs ? 1 : 0);
    auto it = graphs.find(key);
    if (it != graphs.end()) return it->second;
    cudaGraph_t g;
    uint64_t k0 = kcount;
    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < n; ++k) {
      if (mode == MODE_DST)
        launch_step<MODE_DST>(obs && k == 0);
      else
        launch_step<MODE_ICG>(false);
    }
    cudaError_t e = cudaStreamEndCapture(stream, &g);
    graph_kernels[key] = kcount - k0;  // captured, not executed: counted per replay
    kcount = k0;
    if (e != cudaSuccess) throw Error(ST_CUDA, std::string("cuda: ") + cudaGetErrorString(e));
    cudaGraphExec_t ge;
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) throw Error(ST_CUDA, std::string("cuda: ") + cudaGetErrorString(e));
    graphs[key] = ge;
    return ge;
  }

  // Rebuilds the cell grids with per-system cell sides and the per-bead tile
  // size; the state stays on the device and only the cell arrays change.
  // Drops the captured graphs (their launches depend on the kernel choice).
  void graphs_clear() {
    CK(cudaStreamSynchronize(stream));
    for (auto &g : graphs) cudaGraphExecDestroy(g.second);
    graphs.clear();
    graph_kernels.clear();
  }

  void regrid(const std::vector<float> &csl, int new_tile) {
    int64_t total = 0;
    for (size_t s = 0; s < hsys.size(); ++s) total += cells_of(grid_side(geo[s].d_m, csl[s]));
    check_totals(nb, total);
    graphs_clear();
    tile = new_tile;
    nc = 0;
    for (size_t s = 0; s < hsys.size(); ++s) {
      SysDesc &d = hsys[s];
      d.csl = csl[s];
      d.inv_csl = 1.0f / csl[s];
      d.cps = grid_side(geo[s].d_m, csl[s]);
      d.cell_off = nc;
      d.reach = (csl[s] >= need_cut) ? 1 : 2;
      d.cls_cells = typed() ? d.cps * d.cps * d.cps : 0;
      nc += (int)cells_of(d.cps);
    }
    build_tiles();
    nblk = (nc + 1 + SCAN_CHUNK - 1) / SCAN_CHUNK;
    size_t cpad = (size_t)nblk * SCAN_CHUNK;
    counts.alloc(cpad / 4);  // byte counts
    start.alloc(cpad + 4);
    bsum.alloc(nblk + 1);
    lbs_start.alloc(nc + 1);
    d_tiles.alloc(htiles.size());
    d_ctiles.alloc(hctiles.size());
    CK(cudaMemcpyAsync(d_tiles.p, htiles.data(), sizeof(Tile) * htiles.size(),
                       cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_ctiles.p, hctiles.data(), sizeof(Tile) * hctiles.size(),
                       cudaMemcpyHostToDevice, stream));
    CK(cudaMemsetAsync(start.p, 0, sizeof(uint32_t) * (cpad + 4), stream));
    upload_lbs();  // re-sorts the sites into the new cells and uploads hsys
    recount();
    CK(cudaStreamSynchronize(stream));
  }

  // Device ms per Heun step with the current grids (graphs of `reps` steps).
  double time_steps(int reps) {
    run_steps(reps, MODE_DST, 0);  // builds the graph
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, stream));
    run_steps(reps, MODE_DST, 0);
    CK(cudaEventRecord(e1, stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    sync_and_check();
    return ms / reps;
  }

  // Autotuner: for each half-shell pair kernel (2: one grid; 4: the typed
  // layout), per size class (bead counts in [2^k, 2^(k+1))) the cell side
  // factor f (cell side = f * largest cutoff; f >= 1 uses the 3x3x3 stencil,
  // f in [0.5, 1) the 5x5x5 one); then the faster kernel with its cell sides,
  // then the per-bead tile size. Each candidate is timed over `reps` steps;
  // the state, time and noise counter are restored afterwards, so tuning does
  // not change the trajectory. Returns a JSON report.
  std::string autotune(int reps) {
    if (!positions_valid) throw Error(ST_STATE, "positions not initialised");
    if (par.pair_kernel != 2 && par.pair_kernel != 4)
      throw Error(ST_ARG, "autotune needs a half-shell pair kernel");
    download_positions();
    PinnedFloats saved_xyz = hxyz;
    uint64_t saved_step = step;
    const int ns = (int)hsys.size();
    std::vector<int> cls(ns);
    std::map<int, std::vector<int>> members;
    for (int s = 0; s < ns; ++s) {
      int k = 0;
      while ((2 << k) <= hsys[s].n) ++k;
      cls[s] = k;
      members[k].push_back(s);
    }
    std::vector<float> csl0(ns);
    for (int s = 0; s < ns; ++s) csl0[s] = hsys[s].csl;
    const float factors[] = {1.0f, 0.5f, 0.55f, 0.625f, 0.75f};
    struct Choice {
      int kernel;
      double ms;
      std::vector<float> csl;
      std::string classes;
    };
    std::vector<Choice> choices;
    for (int kernel : {par.pair_kernel, par.pair_kernel == 2 ? 4 : 2}) {
      par.pair_kernel = kernel;
      std::vector<float> csl = csl0;
      std::ostringstream rep;
      bool first = true;
      double last = 1e30;
      for (auto &kv : members) {
        double best = 1e30;
        float best_f = 1.0f;
        std::ostringstream tried;
        for (float f : factors) {
          for (int s : kv.second) csl[s] = f * need_cut;
          regrid(csl, tile);
          double ms = time_steps(reps);
          tried << (tried.tellp() > 0 ? ", " : "") << "[" << f << ", " << ms << "]";
          if (ms < best) {
            best = ms;
            best_f = f;
          }
        }
        for (int s : kv.second) csl[s] = best_f * need_cut;
        last = best;
        int nmin = 1 << 30, nmax = 0;
        for (int s : kv.second) {
          nmin = std::min(nmin, hsys[s].n);
          nmax = std::max(nmax, hsys[s].n);
        }
        rep << (first ? "" : ", ") << "{\"n_min\": " << nmin << ", \"n_max\": " << nmax
            << ", \"systems\": " << kv.second.size() << ", \"cell_side\": " << best_f * need_cut
            << ", \"reach\": " << (best_f >= 1.0f ? 1 : 2) << ", \"tried\": [" << tried.str()
            << "]}";
        first = false;
      }
      choices.push_back(Choice{kernel, last, csl, rep.str()});
    }
    const Choice &ch = (choices[1].ms < choices[0].ms) ? choices[1] : choices[0];
    par.pair_kernel = ch.kernel;
    std::vector<float> csl = ch.csl;
    std::ostringstream rep;
    rep << "{\"pair_kernel\": " << ch.kernel << ", \"kernels_tried\": [[" << choices[0].kernel
        << ", " << choices[0].ms << "], [" << choices[1].kernel << ", " << choices[1].ms
        << "]], \"classes\": [" << ch.classes;
    double best = 1e30;
    int best_tile = tile, best_lanes = pair_lanes();
    std::ostringstream tt;
    for (int t : {64, 128, 256}) {
      regrid(csl, t);
      for (int l : {1, 2, 4, 8}) {
        if (t * l > 512) continue;
        par.pair_lanes = l;
        graphs_clear();
        double ms = time_steps(reps);
        tt << (tt.tellp() > 0 ? ", " : "") << "[" << t << ", " << l << ", " << ms << "]";
        if (ms < best) {
          best = ms;
          best_tile = t;
          best_lanes = l;
        }
      }
    }
    par.pair_lanes = best_lanes;
    regrid(csl, best_tile);
    hxyz = saved_xyz;
    upload_positions();
    step = saved_step;
    rep << "], \"tile\": " << best_tile << ", \"lanes\": " << best_lanes
        << ", \"tiles_tried\": [" << tt.str() << "], \"ms_per_step\": " << best << "}";
    return rep.str();
  }

  // Per-kernel device times of `reps` observed steps, each kernel bracketed by
  // its own pair of events on the engine stream.
  void kernel_times(int reps, double *out) {
    if (!positions_valid) throw Error(ST_STATE, "positions not initialised");
    cudaEvent_t e[11];
    for (auto &x : e) CK(cudaEventCreate(&x));
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    set_device_step();
    for (int r = 0; r < reps; ++r) {
      CK(cudaEventRecord(e[0], stream));
      launch_scan(true);
      CK(cudaEventRecord(e[1], stream));
      launch_scatter(pos.p);
      CK(cudaEventRecord(e[2], stream));
      launch_contacts();
      CK(cudaEventRecord(e[3], stream));
      launch_observe();
      CK(cudaEventRecord(e[4], stream));
      launch_pair<MODE_DST>();
      CK(cudaEventRecord(e[5], stream));
      launch_update<1, MODE_DST>();
      CK(cudaEventRecord(e[6], stream));
      launch_scan(false);
      CK(cudaEventRecord(e[7], stream));
      launch_scatter(er.p);
      CK(cudaEventRecord(e[8], stream));
      launch_pair<MODE_DST>();
      CK(cudaEventRecord(e[9], stream));
      launch_update<2, MODE_DST>();
      CK(cudaEventRecord(e[10], stream));
      CK(cudaEventSynchronize(e[10]));
      float t[10];
      for (int k = 0; k < 10; ++k) CK(cudaEventElapsedTime(&t[k], e[k], e[k + 1]));
      acc[0] += 0.5 * (t[0] + t[6]);
      acc[1] += 0.5 * (t[1] + t[7]);
      acc[2] += 0.5 * (t[4] + t[8]);
      acc[3] += t[5];
      acc[4] += t[9];
      acc[5] += t[2];
      acc[6] += t[3];
      ++step;
      ++dev_next;
      ++frames_observed;
    }
    for (auto &x : e) cudaEventDestroy(x);
    for (int k = 0; k < 7; ++k) out[k] = acc[k] / reps;
    sync_and_check();
  }

  // The device counter holds the step being executed; every step's first scan
  // advances it, so it only needs setting when the host moves `step`.
  void set_device_step() {
    if (dev_next == step) return;
    k_set_step<<<1, 1, 0, stream>>>(d_step.p, (unsigned long long)(step - 1));
    CK(cudaGetLastError());
    kcount += 1;
    dev_next = step;
  }

  // n steps of the given mode; observation every obs_every steps (DST only).
  void run_steps(uint64_t n, int mode, uint32_t obs_every) {
    if (!positions_valid) throw Error(ST_STATE, "positions not initialised");
    if (persist_reach > 0) {
      run_steps_persist(n, mode, obs_every);
      return;
    }
    set_device_step();
    const int chunk = 128;
    uint64_t left = n;
    while (left > 0) {
      int g;
      bool obs = false;
      if (mode == MODE_DST && obs_every > 0) {
        uint64_t to_next = (obs_every - (step % obs_every)) % obs_every;
        if (to_next == 0) {
          obs = true;
          g = (int)std::min<uint64_t>(left, obs_every);
        } else {
          g = (int)std::min<uint64_t>(left, to_next);
        }
        if (g > 4 * chunk) g = 4 * chunk;
      } else {
        g = (int)std::min<uint64_t>(left, chunk);
      }
      CK(cudaGraphLaunch(graph_for(mode, g, obs), stream));
      kcount += graph_kernels[std::make_tuple(mode, g, obs ? 1 : 0)];
      if (obs) ++frames_observed;
      step += g;
      dev_next += g;
      left -= g;
    }
  }

  // The persistent path: per chunk (a frame, at most 512 steps) the
  // observation of its first state when due (as the graph path's first step
  // does), one launch of the persistent kernel, and the cell histogram of the
  // new positions that the next sort and observation expect.
  void run_steps_persist(uint64_t n, int mode, uint32_t obs_every) {
    uint64_t left = n;
    while (left > 0) {
      int g;
      bool obs = false;
      if (mode == MODE_DST && obs_every > 0) {
        uint64_t to_next = (obs_every - (step % obs_every)) % obs_every;
        obs = to_next == 0;
        g = (int)std::min<uint64_t>(left, obs ? obs_every : to_next);
      } else {
        g = (int)std::min<uint64_t>(left, 512);
      }
      g = std::min(g, 512);
      if (obs) {
        sort_now();
        launch_observe_sorted(false);
        ++frames_observed;
      }
      launch_persist(mode, g);
      recount();
      step += g;
      left -= g;
    }
    dev_next = ~0ull;  // the device step counter was not advanced
  }

  void sync_and_check() {
    CK(cudaStreamSynchronize(stream));
    int e[ERR_COUNT];
    CK(cudaMemcpy(e, d_err.p, sizeof(e), cudaMemcpyDeviceToHost));
    if (e[ERR_NAN]) throw Error(ST_STATE, "non-finite bead position");
    if (e[ERR_SLOT]) throw Error(ST_STATE, "cell list inconsistent with positions");
  }

  // Standalone analysis at the current positions.
  void sort_now() {
    launch_scan(false);
    launch_scatter(pos.p);
  }

  void observe(bool with_sdist) {
    if (!positions_valid) throw Error(ST_STATE, "positions not initialised");
    sort_now();
    launch_observe_sorted(with_sdist);
    recount();
    CK(cudaGetLastError());
    ++frames_observed;
    sync_and_check();
  }

  void reset_observables() {
    CK(cudaMemsetAsync(map.p, 0, sizeof(int32_t) * std::max<int64_t>(map_total, 1), stream));
    CK(cudaMemsetAsync(ps.p, 0, sizeof(int32_t) * std::max(ps_total, 1), stream));
    CK(cudaMemsetAsync(ds.p, 0, sizeof(double) * std::max(ps_total, 1), stream));
    CK(cudaMemsetAsync(obs.p, 0, sizeof(double) * hsys.size() * OBS_STRIDE, stream));
    frames_observed = 0;
  }

  // One analysis frame of every system at the current positions
  // (chrana::calc_observables, chrana.cu:371-512): the contact map, contact
  // counts and distance sums by separation accumulate in the observable
  // buffers shared with observe(); the per-frame scalars and radial densities
  // are appended to each system's time series.
  void analysis_frame() {
    if (!positions_valid) throw Error(ST_STATE, "positions not initialised");
    const size_t ns = hsys.size();
    if (ana.series.empty()) ana.resize((int)ns);
    if (!fobs.p) {
      fobs.alloc(ns * OBS_STRIDE);
      fextra.alloc(ns * 2);
    }
    sort_now();
    launch_observe_sorted(true);
    CK(cudaMemsetAsync(fobs.p, 0, sizeof(double) * ns * OBS_STRIDE, stream));
    CK(cudaMemsetAsync(fextra.p, 0, sizeof(double) * ns * 2, stream));
    k_observe<<<(unsigned)htiles.size(), tile, 0, stream>>>(d_tiles.p, d_sys.p, pos.p, CCP_RCO / 2.0f, fobs.p);
    k_frame_extra<<<(unsigned)htiles.size(), tile, 0, stream>>>(d_tiles.p, d_sys.p, pos.p, fextra.p);
    kcount += 2;
    recount();
    CK(cudaGetLastError());
    ++frames_observed;
    std::vector<double> fo(ns * OBS_STRIDE), fx(ns * 2);
    CK(cudaMemcpyAsync(fo.data(), fobs.p, sizeof(double) * fo.size(), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(fx.data(), fextra.p, sizeof(double) * fx.size(), cudaMemcpyDeviceToHost, stream));
    sync_and_check();
    std::vector<float> v(ANA_SERIES);
    for (size_t s = 0; s < ns; ++s) {
      const SysDesc &d = hsys[s];
      const double n = d.n;
      const double *o = &fo[s * OBS_STRIDE];
      const double cx = o[0] / n, cy = o[1] / n, cz = o[2] / n, c2 = cx * cx + cy * cy + cz * cz;
      v[0] = (float)std::sqrt(c2);
      v[1] = (float)(o[3] / n - c2);
      v[2] = (float)(fx[2 * s] / (n - 1.0));
      v[3] = (float)(fx[2 * s + 1] / n);
      const double shell = (4.0 / 3.0) * 3.14159265358979323846 * (double)d.R_n * d.R_n * d.R_n / ANA_SHELLS;
      for (int k = 0; k < 3 * ANA_SHELLS; ++k) v[4 + k] = (float)(o[4 + k] / shell);
      ana.add_frame((int)s, v.data());
    }
  }

  // Ends every system's simulation (calc_last_is_stat + clear_is_var,
  // chrana.cu:177-305): frame-averaged spatial distance and contact
  // probability by separation (calc_sd_cp, chrana.cu:13-45) per block and
  // contact-map values (calc_cm, chrana.cu:48-84), statistics of the series,
  // the analysis-XXX.dat text; then the observable buffers are cleared.
  void analysis_end() {
    const int frames = ana.series.empty() ? 0 : ana.frames(0);
    if (frames == 0) throw Error(ST_STATE, "no analysis frame since the simulation began");
    std::vector<int32_t> hmap(std::max<int64_t>(map_total, 1)), hps(std::max(ps_total, 1));
    std::vector<double> hds(std::max(ps_total, 1));
    CK(cudaMemcpyAsync(hmap.data(), map.p, sizeof(int32_t) * hmap.size(), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(hps.data(), ps.p, sizeof(int32_t) * hps.size(), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(hds.data(), ds.p, sizeof(double) * hds.size(), cudaMemcpyDeviceToHost, stream));
    sync_and_check();
    for (size_t s = 0; s < hsys.size(); ++s) {
      const SysDesc &d = hsys[s];
      AnaLayout lay;
      lay.n_beads = d.n;
      lay.R_n = d.R_n;
      // ccp's diploid model: one block per chromosome, both copies together;
      // otherwise one block per chain (at least ccp's six)
      const bool diploid = d.n_copies == 2 && d.n_chains == 12;
      const int nblocks = diploid ? 6 : std::max(ANA_MIN_BLOCKS, d.n_chains);
      lay.block_len.assign(nblocks, 0);
      std::vector<std::vector<double>> sd(nblocks), cp(nblocks);
      for (int blk = 0; blk < nblocks; ++blk) {
        std::vector<int> chains;
        if (diploid) chains = {d.chain_off + blk, d.chain_off + blk + 6};
        else if (blk < d.n_chains) chains = {d.chain_off + blk};
        if (chains.empty()) continue;
        const int L = chain_len[chains[0]], rows = chain_smax[chains[0]];
        lay.block_len[blk] = rows;
        sd[blk].resize(rows);
        cp[blk].resize(rows);
        for (int sep = 1; sep <= rows; ++sep) {
          double cnt = 0.0, dsum = 0.0;
          for (int c : chains) {
            cnt += hps[chain_ps_off[c] + sep];
            dsum += hds[chain_ps_off[c] + sep];
          }
          const double denom = (double)frames * chains.size() * (L - sep);
          cp[blk][sep - 1] = 1000.0 * cnt / denom;
          sd[blk][sep - 1] = dsum / denom;
        }
      }
      const int nb = d.nbins;
      lay.cm_len = (int64_t)nb * (nb + 1) / 2;
      std::vector<double> cm(lay.cm_len);
      const double px = (double)d.map_len / nb;
      for (int bx = 0; bx < nb; ++bx)
        for (int by = 0; by <= bx; ++by) {
          const int64_t k = (int64_t)bx * (bx + 1) / 2 + by;
          const double self = bx == by ? px * d.n_copies : 0.0;
          cm[k] = 1000.0 * (hmap[d.map_off + k] / (double)frames + self) / (d.n_copies * px * px);
        }
      ana.finish((int)s, lay, sd, cp, cm);
    }
    reset_observables();
    sync_and_check();
  }

  std::vector<unsigned long long> overlaps() {
    CK(cudaMemsetAsync(ovl.p, 0, sizeof(unsigned long long) * hsys.size(), stream));
    sort_now();
    launch_contacts_args(contact_args(false, false, true));
    recount();
    CK(cudaGetLastError());
    std::vector<unsigned long long> o(hsys.size());
    CK(cudaMemcpyAsync(o.data(), ovl.p, sizeof(unsigned long long) * o.size(),
                       cudaMemcpyDeviceToHost, stream));
    sync_and_check();
    return o;
  }

  std::vector<float> forces() {
    if (!positions_valid) throw Error(ST_STATE, "positions not initialised");
    sort_now();
    launch_pair<MODE_DST>();
    k_total_force<MODE_DST><<<(unsigned)htiles.size(), tile, 0, stream>>>(
        d_tiles.p, d_sys.p, ff, pos.p, fs.p, rank.p, lbs_sorted.p, lbs_start.p, fout.p);
    recount();
    CK(cudaGetLastError());
    k_pack_xyz<<<(nb + 255) / 256, 256, 0, stream>>>(fout.p, xyz_stage.p, nb);
    std::vector<float> f((size_t)3 * nb);
    CK(cudaMemcpyAsync(f.data(), xyz_stage.p, sizeof(float) * 3 * nb, cudaMemcpyDeviceToHost,
                       stream));
    sync_and_check();
    return f;
  }

  // -------------------------------------------------------------- init
  void generate_initial_condition() {
    for (size_t s = 0; s < hsys.size(); ++s) {
      const SysDesc &d = hsys[s];
      const SystemSpec &q = specs[s];
      HostRng rng(q.seed, 0x51u);
      std::vector<float> l;
      place_lbs(geo[s], ff.lbs_depth, ff.lco, d.n_lbs, rng, l);
      std::copy(l.begin(), l.end(), hlbs.begin() + 3 * (size_t)d.lbs_off);
      std::vector<int32_t> pt;
      if (par.preset == PRESET_CCP)
        make_types_ccp((uint32_t)d.n, par.sequence_file, rng, pt);
      else
        make_types_markov(d.n, par.mean_block, par.lad_fraction, rng, pt);
      std::copy(pt.begin(), pt.end(), hpt.begin() + d.bead_off);
    }
    flags_current = false;
    upload_lbs();
    random_walk(nullptr);
    relax();
    download_positions();
  }

  // Confined random walk of every chain (chrsim::set_particle_positons and
  // perform_random_walk, chrsim.cu:678-802) on the GPU, one warp per chain.
  // ccp's diploid model walks its 12 chromosomes in cones around the 12
  // icosahedral directions, shuffled per system on the host; every other
  // chain walks without a cone. Positions end up in pos (and hxyz); draws, if
  // given, receives each chain's number of attempts.
  void random_walk(uint32_t *draws) {
    std::fill(hxyz.begin(), hxyz.end(), 0.0f);
    upload_positions(false);  // flags; the walk overwrites every position, then counts
    std::vector<WalkChain> wc((size_t)nch);
    for (size_t s = 0; s < hsys.size(); ++s) {
      const SysDesc &d = hsys[s];
      bool diploid = par.preset == PRESET_CCP && (uint32_t)d.n == CCP_N_DEF && d.n_chains == 12;
      const double phi = (1.0 + std::sqrt(5.0)) / 2.0;
      double dir[12][3] = {{0, 1, phi},  {1, phi, 0},  {phi, 0, 1},   {0, 1, -phi},
                           {1, -phi, 0}, {-phi, 0, 1}, {0, -1, phi},  {-1, phi, 0},
                           {phi, 0, -1}, {0, -1, -phi}, {-1, -phi, 0}, {-phi, 0, -1}};
      if (diploid) {  // chrsim.cu:694-703
        HostRng rng(specs[s].seed, 0x52u);
        for (int i = 11; i > 0; --i) {
          float ran = rng.uniform();
          int j = (int)((i + 1) * (1.0 - ran));
          for (int a = 0; a < 3; ++a) std::swap(dir[i][a], dir[j][a]);
        }
      }
      const double mda = diploid ? M_PI / 2.0 - std::atan(phi) : M_PI;
      for (int c = 0; c < d.n_chains; ++c) {
        int g = d.chain_off + c;
        WalkChain &w = wc[g];
        w.first = chain_first[g];
        w.end = (c + 1 < d.n_chains) ? chain_first[g + 1] : d.bead_off + d.n;
        w.k0 = d.seed_lo;
        w.k1 = d.seed_hi;
        w.chain = (uint32_t)c;
        uint64_t budget = 256ull * (uint64_t)(w.end - w.first) + (1ull << 17);
        w.max_draws = (uint32_t)std::min<uint64_t>(budget, 0xFFFFFF00ull);
        w.ax = diploid ? dir[c % 12][0] : 0.0;
        w.ay = diploid ? dir[c % 12][1] : 0.0;
        w.az = diploid ? dir[c % 12][2] : 0.0;
        w.cos_mda = std::cos(mda);
        w.R_n = d.R_n;
      }
    }
    WalkParams wp;
    const double iT = 1.0 / ff.kT;
    const double kb = (ff.k_b > 0.0f) ? ff.k_b : 1.0;
    const double c_b = 0.5 * iT * kb;
    wp.inv_cb = 1.0 / c_b;
    wp.one_m_e = 1.0 - std::exp(-2.0 * c_b);
    wp.l_0 = ff.l_0;
    wp.sig_b = std::sqrt(2.0 / (ff.k_e * iT));
    wp.mis = ff.mis;
    DevBuf<WalkChain> d_wc;
    DevBuf<uint32_t> d_draws;
    DevBuf<double> wxyz;
    d_wc.alloc(std::max<size_t>(wc.size(), 1));
    d_draws.alloc(std::max<size_t>(wc.size(), 1));
    wxyz.alloc((size_t)3 * std::max(nb, 1));
    CK(cudaMemcpyAsync(d_wc.p, wc.data(), sizeof(WalkChain) * wc.size(), cudaMemcpyHostToDevice,
                       stream));
    CK(cudaMemsetAsync(d_err.p + ERR_WALK, 0, sizeof(int), stream));
    k_random_walk<<<(unsigned)((nch + WALK_WARPS - 1) / WALK_WARPS), 32 * WALK_WARPS, 0, stream>>>(
        d_wc.p, nch, wp, pos.p, wxyz.p, d_draws.p, d_err.p);
    CK(cudaGetLastError());
    kcount += 1;
    recount();
    std::vector<uint32_t> used(wc.size());
    CK(cudaMemcpyAsync(used.data(), d_draws.p, sizeof(uint32_t) * used.size(),
                       cudaMemcpyDeviceToHost, stream));
    int e[ERR_COUNT];
    CK(cudaMemcpyAsync(e, d_err.p, sizeof(e), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    if (e[ERR_WALK]) {
      positions_valid = false;
      throw Error(ST_STATE, "confined random walk used up its draw budget");
    }
    if (draws) std::copy(used.begin(), used.end(), draws);
    download_positions();
  }

  // Soft-repulsion relaxation until no non-bonded pair overlaps
  // (chrsim.cu:492-518); rounds of spf steps.
  void relax() {
    for (int round = 0; round < 10000; ++round) {
      auto o = overlaps();
      unsigned long long tot = 0;
      for (auto v : o) tot += v;
      if (tot == 0) return;
      uint64_t saved = step;
      run_steps(par.spf, MODE_ICG, 0);
      step = saved;  // relaxation does not advance simulated time
      sync_and_check();
    }
    throw Error(ST_STATE, "initial condition relaxation did not converge");
  }

  // -------------------------------------------------------------- frames
  // chrsim::run_simulation (chrsim.cu:558-593): fpf frames of spf steps. The
  // steps of frame k+1 are enqueued before the host waits for frame k, so the
  // frame callback (the trajectory write) runs while the GPU computes the next
  // frame. Frame k is packed into fstage[k & 1] on the compute stream and
  // copied to pinned[k & 1] on the copy stream, so the copy does not hold up
  // the next frame's steps either; packing frame k + 2 into the same staging
  // buffer waits for that copy.
  void run_simulation(ccpgpu_frame_fn fn, void *user) {
    if (!positions_valid) throw Error(ST_STATE, "positions not initialised");
    const SysDesc &d0 = hsys[0];
    int pending = -1;
    uint32_t pend_if = 0;
    float pend_t = 0;
    auto deliver = [&](int k) {
      CK(cudaEventSynchronize(ev[k]));
      if (fn && fn(user, pend_if, pend_t, pinned[k] + 3 * (size_t)d0.bead_off, d0.n)) {
        CK(cudaStreamSynchronize(cstream));
        CK(cudaStreamSynchronize(stream));
        throw Error(ST_IO, "frame callback failed");
      }
    };
    for (uint32_t ffi = 0; ffi < par.fpf; ++ffi) {
      run_steps(par.spf, MODE_DST, 0);
      int b = ffi & 1;
      if (ffi >= 2) CK(cudaStreamWaitEvent(stream, ev[b], 0));
      k_pack_xyz<<<(nb + 255) / 256, 256, 0, stream>>>(pos.p, fstage[b].p, nb);
      CK(cudaGetLastError());
      CK(cudaEventRecord(ev_pack[b], stream));
      CK(cudaStreamWaitEvent(cstream, ev_pack[b], 0));
      CK(cudaMemcpyAsync(pinned[b], fstage[b].p, sizeof(float) * 3 * nb, cudaMemcpyDeviceToHost,
                         cstream));
      CK(cudaEventRecord(ev[b], cstream));
      for (auto &v : i_f) ++v;
      for (auto &v : t) v += par.spf * ff.dt;
      if (pending >= 0) deliver(pending);
      pending = b;
      pend_if = i_f[0];
      pend_t = t[0];
    }
    if (pending >= 0) {
      deliver(pending);
      std::memcpy(hxyz.data(), pinned[pending], sizeof(float) * 3 * nb);
    }
    sync_and_check();
  }
};

// ------------------------------------------------------------------ helpers

static std::vector<SystemSpec> single_spec(const Params &p, uint64_t seed) {
  SystemSpec s;
  s.n = (int)p.N;
  s.R_n = p.R_n;
  s.R_o = p.R_o;
  s.R_b = p.R_b;
  s.n_lbs = (int)p.n_l;
  s.seed = seed;
  s.contact_bins = p.contact_bins;
  if (p.preset == PRESET_CCP && p.N == CCP_N_DEF && p.n_chains == 12) {
    for (int c = 0; c < 12; ++c) s.chain_first.push_back((int)CCP_CHR_LIM[c]);
    s.n_chains = 12;
  } else {
    s.n_chains = p.n_chains;
  }
  return {s};
}

}  // namespace ccpgpu

using namespace ccpgpu;

struct ccpgpu_sim {
  std::unique_ptr<Engine> e;
};

static thread_local std::string g_last_error;

void ccpgpu::set_last_error(const std::string &m) { g_last_error = m; }

template <typename F>
static int guarded(F &&f) {
  try {
    f();
    return CCPGPU_OK;
  } catch (const Error &e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc &) {
    g_last_error = "out of host memory";
    return CCPGPU_ERR_ARG;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return CCPGPU_ERR_ARG;
  }
}

static void need(bool c, const char *m) {
  if (!c) throw Error(ST_ARG, m);
}

static int put_bytes(const std::string &s, void *buf, size_t cap, size_t *len) {
  if (len) *len = s.size();
  if (!buf || cap < s.size()) {
    g_last_error = "buffer too small";
    return CCPGPU_ERR_IO;
  }
  std::memcpy(buf, s.data(), s.size());
  return CCPGPU_OK;
}

extern "C" {

const char *ccpgpu_last_error(void) { return g_last_error.c_str(); }

int ccpgpu_create(const char *param_text, uint64_t seed, ccpgpu_sim **out) {
  return guarded([&] {
    need(param_text && out, "null argument");
    *out = nullptr;
    Params p = parse_params(param_text);
    uint64_t sd = ParamMap(param_text).has("seed") ? p.seed : seed;
    auto h = std::make_unique<ccpgpu_sim>();
    h->e = std::make_unique<Engine>();
    h->e->build(p, single_spec(p, sd));
    *out = h.release();
  });
}

int ccpgpu_batch_create(const char *param_text, int32_t n_systems, const int32_t *n_beads,
                        const int32_t *n_chains, const float *radii, const uint64_t *seeds,
                        uint64_t seed, ccpgpu_sim **out) {
  return guarded([&] {
    need(param_text && out && n_beads && n_systems > 0, "null argument");
    *out = nullptr;
    Params p = parse_params(param_text);
    ParamMap pm(param_text);
    std::vector<SystemSpec> sp(n_systems);
    for (int s = 0; s < n_systems; ++s) {
      SystemSpec &q = sp[s];
      q.n = n_beads[s];
      need(q.n >= 1, "system without beads");
      const bool diploid_size = p.preset == PRESET_CCP && (uint32_t)q.n == CCP_N_DEF;
      if (n_chains)
        q.n_chains = n_chains[s];
      else if (pm.has("number_of_chains"))
        q.n_chains = p.n_chains;
      else
        q.n_chains = diploid_size ? 12 : 1;
      need(q.n_chains >= 1 && q.n_chains <= q.n, "bad chain count");
      // ccp's diploid model: 12 chromosomes at its fixed limits (chrdat.cuh:28-31),
      // as a single system created from the same text
      if (diploid_size && q.n_chains == 12)
        for (int c = 0; c < 12; ++c) q.chain_first.push_back((int)CCP_CHR_LIM[c]);
      if (radii)
        q.R_n = radii[s];
      else if (pm.has("nucleus_radius"))
        q.R_n = p.R_n;
      else
        q.R_n = (float)(0.5 * std::cbrt((double)q.n / p.packing_fraction));
      need(q.R_n > 1.0f, "nucleus radius too small");
      q.R_o = 0.0f;
      q.R_b = 0.0f;
      Geometry g = make_geometry(q.R_n, q.R_o, q.R_b);
      if (pm.has("number_of_lbs")) {
        q.n_lbs = (int)p.n_l;
      } else if (p.preset == PRESET_BASELINE) {
        float noacf = 2.0f / (1.0f + g.noc);
        q.n_lbs = (int)std::floor(p.lbs_area_fraction * 4.0 /
                                  std::pow(p.ff.lco / (q.R_n - p.ff.lbs_depth), 2.0) * noacf);
      } else {
        q.n_lbs = 0;
      }
      q.seed = seeds ? seeds[s] : (seed + (uint64_t)s);
      q.contact_bins = p.contact_bins;
    }
    auto h = std::make_unique<ccpgpu_sim>();
    h->e = std::make_unique<Engine>();
    h->e->build(p, std::move(sp));
    *out = h.release();
  });
}

int ccpgpu_destroy(ccpgpu_sim *h) {
  return guarded([&] { delete h; });
}

int ccpgpu_info_get(const ccpgpu_sim *h, ccpgpu_info *o) {
  return guarded([&] {
    need(h && o, "null argument");
    const Engine &e = *h->e;
    std::memset(o, 0, sizeof(*o));
    o->n_systems = (int32_t)e.hsys.size();
    o->n_beads = e.nb;
    o->n_lbs = e.nl;
    o->n_chains = e.nch;
    o->n_cells = e.nc;
    o->preset = e.par.preset;
    o->frames_per_file = e.par.fpf;
    o->steps_per_frame = e.par.spf;
    o->frame_index = e.i_f[0];
    o->time = e.t[0];
    o->step = e.step;
    o->dt = e.ff.dt;
    o->kT = e.ff.kT;
    o->noise_sd = e.ff.sd;
    o->contact_cutoff = e.par.contact_cutoff;
    o->frames_observed = e.frames_observed;
    o->persistent_reach = e.persist_reach;
  });
}

int ccpgpu_system_info_get(const ccpgpu_sim *h, int32_t sys, ccpgpu_system_info *o) {
  return guarded([&] {
    need(h && o, "null argument");
    const Engine &e = *h->e;
    need(sys >= 0 && sys < (int)e.hsys.size(), "system index out of range");
    const SysDesc &d = e.hsys[sys];
    std::memset(o, 0, sizeof(*o));
    o->bead_offset = d.bead_off;
    o->n_beads = d.n;
    o->chain_offset = d.chain_off;
    o->n_chains = d.n_chains;
    o->lbs_offset = d.lbs_off;
    o->n_lbs = d.n_lbs;
    o->cells_per_side = d.cps;
    o->cell_side = d.csl;
    o->nucleus_radius = d.R_n;
    o->opening_radius = d.R_o;
    o->bleb_radius = d.R_b;
    o->contact_bins = d.nbins;
    o->map_len = d.map_len;
    o->copy_len = d.copy_len;
    o->n_copies = d.n_copies;
    o->map_offset = d.map_off;
    o->seed = e.specs[sys].seed;
  });
}

int ccpgpu_generate_initial_condition(ccpgpu_sim *h) {
  return guarded([&] {
    need(h, "null argument");
    h->e->generate_initial_condition();
  });
}

int ccpgpu_random_walk(ccpgpu_sim *h, uint32_t *draws, size_t n) {
  return guarded([&] {
    need(h, "null argument");
    need(!draws || n >= (size_t)h->e->nch, "buffer too small");
    h->e->random_walk(draws);
  });
}

int ccpgpu_run_simulation(ccpgpu_sim *h, ccpgpu_frame_fn fn, void *user) {
  return guarded([&] {
    need(h, "null argument");
    h->e->run_simulation(fn, user);
  });
}

int ccpgpu_run_steps(ccpgpu_sim *h, uint64_t n_steps, uint32_t observe_every) {
  return guarded([&] {
    need(h, "null argument");
    Engine &e = *h->e;
    e.run_steps(n_steps, MODE_DST, observe_every);
    e.sync_and_check();
    e.download_positions();
  });
}

int ccpgpu_advance(ccpgpu_sim *h, uint64_t n_steps, uint32_t observe_every) {
  return guarded([&] {
    need(h, "null argument");
    h->e->run_steps(n_steps, MODE_DST, observe_every);
  });
}

int ccpgpu_synchronize(ccpgpu_sim *h) {
  return guarded([&] {
    need(h, "null argument");
    h->e->sync_and_check();
  });
}

int ccpgpu_stream_handle(ccpgpu_sim *h, void **stream) {
  return guarded([&] {
    need(h && stream, "null argument");
    *stream = (void *)h->e->stream;
  });
}

int ccpgpu_kernel_times(ccpgpu_sim *h, int32_t reps, double *out, size_t n) {
  return guarded([&] {
    need(h && out && reps > 0, "null argument");
    need(n >= 7, "buffer too small");
    h->e->kernel_times(reps, out);
  });
}

int ccpgpu_autotune(ccpgpu_sim *h, int32_t reps, char *report, size_t cap, size_t *len) {
  int rc = CCPGPU_OK;
  int g = guarded([&] {
    need(h && reps > 0, "null argument");
    std::string r = h->e->autotune(reps);
    rc = put_bytes(r + std::string(1, '\0'), report, cap, len);
  });
  return g ? g : rc;
}

int ccpgpu_kernel_count(const ccpgpu_sim *h, uint64_t *count) {
  return guarded([&] {
    need(h && count, "null argument");
    *count = h->e->kcount;
  });
}

int ccpgpu_error_flags(ccpgpu_sim *h, int32_t *flags8, int32_t clear) {
  return guarded([&] {
    need(h && flags8, "null argument");
    Engine &e = *h->e;
    CK(cudaStreamSynchronize(e.stream));
    CK(cudaMemcpy(flags8, e.d_err.p, sizeof(int) * ERR_COUNT, cudaMemcpyDeviceToHost));
    if (clear) CK(cudaMemset(e.d_err.p, 0, sizeof(int) * ERR_COUNT));
    if (flags8[ERR_NAN] || flags8[ERR_SLOT]) throw Error(ST_STATE, "device error flag set");
  });
}

int ccpgpu_get_positions(ccpgpu_sim *h, float *xyz, size_t n) {
  return guarded([&] {
    need(h && xyz, "null argument");
    Engine &e = *h->e;
    need(n >= (size_t)3 * e.nb, "buffer too small");
    if (e.positions_valid) e.download_positions();
    host_copy(xyz, e.hxyz.data(), sizeof(float) * 3 * e.nb);
  });
}

int ccpgpu_set_positions(ccpgpu_sim *h, const float *xyz, size_t n) {
  return guarded([&] {
    need(h && xyz, "null argument");
    Engine &e = *h->e;
    need(n >= (size_t)3 * e.nb, "buffer too small");
    host_copy(e.hxyz.data(), xyz, sizeof(float) * 3 * e.nb);
    if (!e.lbs_uploaded) e.upload_lbs();
    e.upload_xyz();
  });
}

int ccpgpu_get_types(const ccpgpu_sim *h, int32_t *pt, size_t n) {
  return guarded([&] {
    need(h && pt, "null argument");
    need(n >= (size_t)h->e->nb, "buffer too small");
    std::memcpy(pt, h->e->hpt.data(), 4 * (size_t)h->e->nb);
  });
}

int ccpgpu_set_types(ccpgpu_sim *h, const int32_t *pt, size_t n) {
  return guarded([&] {
    need(h && pt, "null argument");
    Engine &e = *h->e;
    need(n >= (size_t)e.nb, "buffer too small");
    std::memcpy(e.hpt.data(), pt, 4 * (size_t)e.nb);
    e.flags_current = false;
    if (e.positions_valid) {
      e.download_positions();
      e.upload_positions();
    }
  });
}

int ccpgpu_get_lbs(const ccpgpu_sim *h, float *xyz, size_t n) {
  return guarded([&] {
    need(h && (xyz || h->e->nl == 0), "null argument");
    need(n >= (size_t)3 * h->e->nl, "buffer too small");
    if (h->e->nl) std::memcpy(xyz, h->e->hlbs.data(), sizeof(float) * 3 * h->e->nl);
  });
}

int ccpgpu_set_lbs(ccpgpu_sim *h, const float *xyz, size_t n) {
  return guarded([&] {
    need(h && (xyz || h->e->nl == 0), "null argument");
    Engine &e = *h->e;
    need(n >= (size_t)3 * e.nl, "buffer too small");
    if (e.nl) std::memcpy(e.hlbs.data(), xyz, sizeof(float) * 3 * e.nl);
    e.upload_lbs();
  });
}

int ccpgpu_compute_forces(ccpgpu_sim *h, float *f, size_t n) {
  return guarded([&] {
    need(h && f, "null argument");
    Engine &e = *h->e;
    need(n >= (size_t)3 * e.nb, "buffer too small");
    auto v = e.forces();
    std::memcpy(f, v.data(), sizeof(float) * 3 * e.nb);
  });
}

static const SysDesc &sys_of(ccpgpu_sim *h, int32_t sys) {
  need(sys >= 0 && sys < (int)h->e->hsys.size(), "system index out of range");
  return h->e->hsys[sys];
}

int ccpgpu_frame_txt(ccpgpu_sim *h, int32_t sys, char *buf, size_t cap, size_t *len) {
  int rc = CCPGPU_OK;
  int g = guarded([&] {
    need(h, "null argument");
    Engine &e = *h->e;
    const SysDesc &d = sys_of(h, sys);
    if (e.positions_valid) e.download_positions();
    std::vector<int32_t> pt(e.hpt.begin() + d.bead_off, e.hpt.begin() + d.bead_off + d.n);
    rc = put_bytes(format_frame_txt(e.i_f[sys], e.t[sys], pt, e.hxyz.data() + 3 * (size_t)d.bead_off,
                                    d.n),
                   buf, cap, len);
  });
  return g ? g : rc;
}

int ccpgpu_lbs_txt(ccpgpu_sim *h, int32_t sys, char *buf, size_t cap, size_t *len) {
  int rc = CCPGPU_OK;
  int g = guarded([&] {
    need(h, "null argument");
    Engine &e = *h->e;
    const SysDesc &d = sys_of(h, sys);
    rc = put_bytes(format_lbs_txt(e.hlbs.data() + 3 * (size_t)d.lbs_off, d.n_lbs), buf, cap, len);
  });
  return g ? g : rc;
}

int ccpgpu_frame_trr(ccpgpu_sim *h, int32_t sys, char *buf, size_t cap, size_t *len) {
  int rc = CCPGPU_OK;
  int g = guarded([&] {
    need(h, "null argument");
    Engine &e = *h->e;
    const SysDesc &d = sys_of(h, sys);
    if (e.positions_valid) e.download_positions();
    rc = put_bytes(
        format_trr_frame(e.i_f[sys], e.t[sys], e.hxyz.data() + 3 * (size_t)d.bead_off, d.n), buf,
        cap, len);
  });
  return g ? g : rc;
}

int ccpgpu_checkpoint(ccpgpu_sim *h, int32_t sys, void *buf, size_t cap, size_t *len) {
  int rc = CCPGPU_OK;
  int g = guarded([&] {
    need(h, "null argument");
    Engine &e = *h->e;
    const SysDesc &d = sys_of(h, sys);
    if (e.positions_valid) e.download_positions();
    std::vector<int32_t> pt(e.hpt.begin() + d.bead_off, e.hpt.begin() + d.bead_off + d.n);
    rc = put_bytes(format_checkpoint(e.i_f[sys], e.t[sys], pt,
                                     e.hxyz.data() + 3 * (size_t)d.bead_off, d.n,
                                     e.hlbs.data() + 3 * (size_t)d.lbs_off, d.n_lbs),
                   buf, cap, len);
  });
  return g ? g : rc;
}

int ccpgpu_load_checkpoint(ccpgpu_sim *h, int32_t sys, const void *buf, size_t len) {
  return guarded([&] {
    need(h && buf, "null argument");
    Engine &e = *h->e;
    const SysDesc &d = sys_of(h, sys);
    uint32_t i_f;
    float t;
    std::vector<int32_t> pt;
    std::vector<float> x, l;
    if (!parse_checkpoint(buf, len, d.n, d.n_lbs, i_f, t, pt, x, l))
      throw Error(ST_IO, "failed to read checkpoint");
    if (e.positions_valid) e.download_positions();
    std::copy(pt.begin(), pt.end(), e.hpt.begin() + d.bead_off);
    e.flags_current = false;
    std::copy(x.begin(), x.end(), e.hxyz.begin() + 3 * (size_t)d.bead_off);
    std::copy(l.begin(), l.end(), e.hlbs.begin() + 3 * (size_t)d.lbs_off);
    e.i_f[sys] = i_f;
    e.t[sys] = t;
    // noise continues from the step implied by the frame index
    e.step = (uint64_t)i_f * e.par.spf;
    e.upload_lbs();
    e.upload_positions();
  });
}

int ccpgpu_read_frame_txt(ccpgpu_sim *h, int32_t sys, const char *text, size_t len) {
  return guarded([&] {
    need(h && text, "null argument");
    Engine &e = *h->e;
    const SysDesc &d = sys_of(h, sys);
    uint32_t i_f;
    float t;
    std::vector<int32_t> pt;
    std::vector<float> x;
    if (!parse_frame_txt(std::string(text, len), d.n, i_f, t, pt, x))
      throw Error(ST_IO, "failed to read frame from text file");
    if (e.positions_valid) e.download_positions();
    std::copy(pt.begin(), pt.end(), e.hpt.begin() + d.bead_off);
    e.flags_current = false;
    std::copy(x.begin(), x.end(), e.hxyz.begin() + 3 * (size_t)d.bead_off);
    e.i_f[sys] = i_f;
    e.t[sys] = t;
    e.upload_lbs();
    e.upload_positions();
  });
}

int ccpgpu_read_lbs_txt(ccpgpu_sim *h, int32_t sys, const char *text, size_t len) {
  return guarded([&] {
    need(h && text, "null argument");
    Engine &e = *h->e;
    const SysDesc &d = sys_of(h, sys);
    std::vector<float> l;
    if (!parse_lbs_txt(std::string(text, len), d.n_lbs, l))
      throw Error(ST_IO, "failed to read lamina binding sites from text file");
    std::copy(l.begin(), l.end(), e.hlbs.begin() + 3 * (size_t)d.lbs_off);
    e.upload_lbs();
  });
}

int ccpgpu_observe(ccpgpu_sim *h, int32_t with_sdist) {
  return guarded([&] {
    need(h, "null argument");
    h->e->observe(with_sdist != 0);
  });
}

int ccpgpu_analysis_frame(ccpgpu_sim *h) {
  return guarded([&] {
    need(h, "null argument");
    h->e->analysis_frame();
  });
}

int ccpgpu_analysis_series(ccpgpu_sim *h, int32_t sys, float *out, size_t n, int32_t *frames) {
  return guarded([&] {
    need(h && frames, "null argument");
    sys_of(h, sys);
    const Engine &e = *h->e;
    const int f = e.ana.series.empty() ? 0 : e.ana.frames(sys);
    *frames = f;
    if (!out) return;
    need(n >= (size_t)ANA_SERIES * f, "buffer too small");
    for (int k = 0; k < ANA_SERIES; ++k)
      std::copy(e.ana.series[sys][k].begin(), e.ana.series[sys][k].end(), out + (size_t)k * f);
  });
}

int ccpgpu_analysis_end_simulation(ccpgpu_sim *h) {
  return guarded([&] {
    need(h, "null argument");
    h->e->analysis_end();
  });
}

int ccpgpu_analysis_txt(ccpgpu_sim *h, int32_t sys, char *buf, size_t cap, size_t *len) {
  int rc = CCPGPU_OK;
  int g = guarded([&] {
    need(h, "null argument");
    sys_of(h, sys);
    const Engine &e = *h->e;
    if (e.ana.last_txt.empty() || e.ana.last_txt[sys].empty())
      throw Error(ST_STATE, "no finished analysis simulation");
    rc = put_bytes(e.ana.last_txt[sys], buf, cap, len);
  });
  return g ? g : rc;
}

int ccpgpu_analysis_fin_txt(ccpgpu_sim *h, char *buf, size_t cap, size_t *len) {
  int rc = CCPGPU_OK;
  int g = guarded([&] {
    need(h, "null argument");
    rc = put_bytes(h->e->ana.final_txt(), buf, cap, len);
  });
  return g ? g : rc;
}

int ccpgpu_contact_map_bin(ccpgpu_sim *h, char *buf, size_t cap, size_t *len) {
  int rc = CCPGPU_OK;
  int g = guarded([&] {
    need(h, "null argument");
    rc = put_bytes(h->e->ana.contact_map_bin(), buf, cap, len);
  });
  return g ? g : rc;
}

int ccpgpu_reset_observables(ccpgpu_sim *h) {
  return guarded([&] {
    need(h, "null argument");
    h->e->reset_observables();
    CK(cudaStreamSynchronize(h->e->stream));
  });
}

int ccpgpu_contact_counts(ccpgpu_sim *h, int32_t sys, int32_t *tri, size_t n) {
  return guarded([&] {
    need(h && tri, "null argument");
    Engine &e = *h->e;
    const SysDesc &d = sys_of(h, sys);
    size_t m = (size_t)d.nbins * (d.nbins + 1) / 2;
    need(n >= m, "buffer too small");
    CK(cudaStreamSynchronize(e.stream));
    CK(cudaMemcpy(tri, e.map.p + d.map_off, sizeof(int32_t) * m, cudaMemcpyDeviceToHost));
  });
}

int ccpgpu_observable_sums(ccpgpu_sim *h, int32_t sys, double *out, size_t n) {
  return guarded([&] {
    need(h && out, "null argument");
    Engine &e = *h->e;
    sys_of(h, sys);
    need(n >= (size_t)OBS_STRIDE, "buffer too small");
    CK(cudaStreamSynchronize(e.stream));
    CK(cudaMemcpy(out, e.obs.p + (size_t)sys * OBS_STRIDE, sizeof(double) * OBS_STRIDE,
                  cudaMemcpyDeviceToHost));
  });
}

int ccpgpu_separation_counts(ccpgpu_sim *h, int32_t chain, int32_t *counts, double *dist,
                             size_t n) {
  return guarded([&] {
    need(h, "null argument");
    Engine &e = *h->e;
    need(chain >= 0 && chain < e.nch, "chain index out of range");
    size_t m = (size_t)e.chain_smax[chain] + 1;
    need(n >= m, "buffer too small");
    CK(cudaStreamSynchronize(e.stream));
    if (counts)
      CK(cudaMemcpy(counts, e.ps.p + e.chain_ps_off[chain], sizeof(int32_t) * m,
                    cudaMemcpyDeviceToHost));
    if (dist)
      CK(cudaMemcpy(dist, e.ds.p + e.chain_ps_off[chain], sizeof(double) * m,
                    cudaMemcpyDeviceToHost));
  });
}

int ccpgpu_overlaps(ccpgpu_sim *h, uint64_t *per_system, size_t n) {
  return guarded([&] {
    need(h && per_system, "null argument");
    Engine &e = *h->e;
    need(n >= e.hsys.size(), "buffer too small");
    auto o = e.overlaps();
    for (size_t s = 0; s < o.size(); ++s) per_system[s] = o[s];
  });
}

}  // extern "C"

// ====================================================================== no-allocation forces
//
// Some callers cannot allocate device memory at the moment they need forces:
// a host whose memory manager owns all of the GPU's memory and forbids foreign
// cudaMalloc, or a time-critical loop where the implicit device
// synchronisation of cudaMalloc/cudaFree would stall its other streams.
// ccpgpu_forces_noalloc serves them: it evaluates the total force of one
// system from caller-provided device buffers, and its cell list, cell-ordered
// copy and force scratch live in one fixed static device array instead of
// memory allocated per handle.

namespace ccpgpu {
namespace noalloc {

constexpr int MAX_BEADS = CCPGPU_NOALLOC_MAX_BEADS;
constexpr int MAX_CELLS = CCPGPU_NOALLOC_MAX_CELLS;
constexpr int SCAN_CELLS = ((MAX_CELLS + 1 + SCAN_CHUNK - 1) / SCAN_CHUNK) * SCAN_CHUNK;
constexpr int SCAN_BLOCKS = SCAN_CELLS / SCAN_CHUNK;
constexpr int MAX_TILES = (MAX_BEADS + TILE - 1) / TILE;

// byte layout of the scratch array (each part 256-byte aligned)
constexpr size_t al(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t OFF_POS = 0;
constexpr size_t OFF_SORTED = OFF_POS + al(sizeof(float4) * (MAX_BEADS + 1));
constexpr size_t OFF_FS = OFF_SORTED + al(sizeof(float4) * (MAX_BEADS + 1));
constexpr size_t OFF_FOUT = OFF_FS + al(sizeof(float4) * (MAX_BEADS + 1));
constexpr size_t OFF_RANK = OFF_FOUT + al(sizeof(float4) * (MAX_BEADS + 1));
constexpr size_t OFF_COUNTS = OFF_RANK + al(sizeof(uint32_t) * (MAX_BEADS + 1));
constexpr size_t OFF_START = OFF_COUNTS + al(SCAN_CELLS);  // one byte count per cell
constexpr size_t OFF_BSUM = OFF_START + al(sizeof(uint32_t) * (SCAN_CELLS + 4));
constexpr size_t OFF_TILES = OFF_BSUM + al(sizeof(uint32_t) * (SCAN_BLOCKS + 1));
constexpr size_t OFF_SYS = OFF_TILES + al(sizeof(Tile) * MAX_TILES);
constexpr size_t OFF_STEP = OFF_SYS + al(sizeof(SysDesc));
constexpr size_t OFF_ERR = OFF_STEP + al(sizeof(unsigned long long));
constexpr size_t BYTES = OFF_ERR + al(sizeof(int) * ERR_COUNT);

// The scratch: about 2.9 MB, held by every GPU that loads the library until
// the process exits. Device code could name it directly; host code only knows
// its host-side stand-in and obtains the device address per device below.
static __device__ __align__(256) unsigned char scratch[BYTES];

constexpr int MAX_DEVICES = 64;
static std::mutex g_mutex;
static unsigned char *g_base[MAX_DEVICES] = {};

// Device address of the scratch array on the current device, looked up once
// per device with that device current.
static unsigned char *scratch_base(int dev) {
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_base[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, scratch);
    if (e != cudaSuccess) throw Error(ST_CUDA, std::string("cuda: ") + cudaGetErrorString(e));
    g_base[dev] = static_cast<unsigned char *>(p);
  }
  return g_base[dev];
}

// Writes the system descriptor and the bead tiles of the single system.
__global__ void k_na_setup(SysDesc d, Tile *tiles, SysDesc *sys, int n_tiles) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *sys = d;
  if (i < n_tiles) tiles[i] = Tile{0, i * TILE};
}

// Packed xyz + ccp type codes -> float4 positions with the bead flags of the
// preset; n_chains chain heads at c * L, L = n / n_chains, the last chain
// taking the remainder (as the allocating engine places them).
__global__ void k_na_pack(const float *__restrict__ xyz, const int32_t *__restrict__ pt, int n,
                          int chain_len, int n_chains, int preset, float4 *__restrict__ pos,
                          int *__restrict__ err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  uint32_t f = BF_START;
  float x = 0.0f, y = 0.0f, z = 0.0f;
  if (i < n) {
    f = 0u;
    bool a = (pt[i] & 1) == 0;
    if (a) f |= BF_HET;
    if (preset == PRESET_CCP ? a : ((pt[i] & 2) != 0)) f |= BF_LAD;
    if (i % chain_len == 0 && i / chain_len < n_chains) f |= BF_START;
    x = xyz[3 * i];
    y = xyz[3 * i + 1];
    z = xyz[3 * i + 2];
    if (!(isfinite(x) && isfinite(y) && isfinite(z))) set_err(err, ERR_NAN);
  }
  pos[i] = make_float4(x, y, z, __uint_as_float(f));
}

}  // namespace noalloc
}  // namespace ccpgpu

extern "C" int ccpgpu_forces_noalloc(const ccpgpu_noalloc_system *sysp, const float *d_xyz,
                                     const int32_t *d_types, float *d_forces, void *stream) {
  using namespace ccpgpu::noalloc;
  return guarded([&] {
    need(sysp && d_xyz && d_types && d_forces, "null argument");
    const ccpgpu_noalloc_system a = *sysp;
    need(a.preset == PRESET_CCP || a.preset == PRESET_BASELINE, "preset out of range");
    if (!(a.n_beads >= 3 && a.n_beads <= MAX_BEADS))
      throw Error(ST_ARG, "n_beads outside 3.." + std::to_string(MAX_BEADS) +
                              " (the no-allocation scratch limit)");
    need(a.n_chains >= 1 && a.n_chains <= a.n_beads, "bad chain count");
    need(std::isfinite(a.nucleus_radius) && a.nucleus_radius > 1.0f,
         "nucleus radius not finite or too small");
    // the preset force field and cell grid (as parse_params sets them)
    ForceField ff = make_preset(a.preset);
    const float csl = (a.preset == PRESET_CCP) ? CCP_ACO : std::max(ff.rc_att, 1.5f);
    Geometry g = make_geometry(a.nucleus_radius, 0.0f, 0.0f);
    SysDesc d{};
    d.bead_off = 0;
    d.n = a.n_beads;
    d.csl = csl;
    d.inv_csl = 1.0f / csl;
    // bound the half side in float before it becomes an int: the grid of the
    // largest allowed nucleus is far below this, so only the cell limit applies
    const float half = std::ceil(g.d_m / csl);
    if (!(half <= 64.0f))
      throw Error(ST_ARG, "cell grid exceeds the " + std::to_string(MAX_CELLS) +
                              "-cell no-allocation limit");
    d.cps = std::max(2, 2 * (int)half);
    long long cells = (long long)d.cps * d.cps * d.cps;
    if (cells > MAX_CELLS)
      throw Error(ST_ARG, "cell grid of " + std::to_string(cells) + " cells exceeds the " +
                              std::to_string(MAX_CELLS) + "-cell no-allocation limit");
    d.cell_off = 0;
    d.R_n = g.R_n;
    d.R_o = g.R_o;
    d.R_b = g.R_b;
    d.noc = g.noc;
    d.boc = g.boc;
    d.nod = g.nod;
    d.bod = g.bod;
    d.n_lbs = 0;
    d.lbs_rmin = 1e30f;
    d.lbs_rmax = -1e30f;
    d.n_chains = a.n_chains;
    const int nc = (int)cells;
    const int nblk = (nc + 1 + SCAN_CHUNK - 1) / SCAN_CHUNK;
    const int n_tiles = (a.n_beads + TILE - 1) / TILE;

    int dev = 0;
    CK(cudaGetDevice(&dev));
    need(dev >= 0 && dev < MAX_DEVICES, "device index out of range");
    unsigned char *base = scratch_base(dev);
    float4 *pos = reinterpret_cast<float4 *>(base + OFF_POS);
    float4 *sorted = reinterpret_cast<float4 *>(base + OFF_SORTED);
    float4 *fs = reinterpret_cast<float4 *>(base + OFF_FS);
    float4 *fout = reinterpret_cast<float4 *>(base + OFF_FOUT);
    uint32_t *rank = reinterpret_cast<uint32_t *>(base + OFF_RANK);
    uint32_t *counts = reinterpret_cast<uint32_t *>(base + OFF_COUNTS);
    uint32_t *start = reinterpret_cast<uint32_t *>(base + OFF_START);
    uint32_t *bsum = reinterpret_cast<uint32_t *>(base + OFF_BSUM);
    Tile *tiles = reinterpret_cast<Tile *>(base + OFF_TILES);
    SysDesc *sys = reinterpret_cast<SysDesc *>(base + OFF_SYS);
    unsigned long long *step = reinterpret_cast<unsigned long long *>(base + OFF_STEP);
    int *err = reinterpret_cast<int *>(base + OFF_ERR);
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    // the array keeps the previous call's contents: clear what must start at zero
    CK(cudaMemsetAsync(counts, 0, (size_t)nblk * SCAN_CHUNK, s));  // byte counts
    CK(cudaMemsetAsync(err, 0, sizeof(int) * ERR_COUNT, s));
    k_na_setup<<<(n_tiles + 127) / 128, 128, 0, s>>>(d, tiles, sys, n_tiles);
    k_na_pack<<<(a.n_beads + 1 + 255) / 256, 256, 0, s>>>(
        d_xyz, d_types, a.n_beads, a.n_beads / a.n_chains, a.n_chains, a.preset, pos, err);
    k_count<<<n_tiles, TILE, 0, s>>>(tiles, sys, pos, counts, rank, err);
    k_scan_reduce<<<nblk, SCAN_THREADS, 0, s>>>(counts, bsum);
    k_scan_top<<<1, SCAN_TOP_THREADS, 0, s>>>(bsum, nblk, step, 0);
    k_scan_apply<<<nblk, SCAN_THREADS, 0, s>>>(counts, bsum, start, nc, nblk);
    k_scatter<<<n_tiles, TILE, 0, s>>>(tiles, sys, pos, rank, start, sorted, fs, counts, err);
    k_pair_half<MODE_DST><<<n_tiles, TILE, 0, s>>>(tiles, sys, ff, sorted, start, fs);
    k_total_force<MODE_DST><<<n_tiles, TILE, 0, s>>>(tiles, sys, ff, pos, fs, rank, nullptr,
                                                     nullptr, fout);
    k_pack_xyz<<<(a.n_beads + 255) / 256, 256, 0, s>>>(fout, d_forces, a.n_beads);
    CK(cudaGetLastError());
  });
}

// Device flags of the last ccpgpu_forces_noalloc call on the current device,
// read after the caller's stream has finished that call. Non-finite positions
// and inconsistent cell slots are reported as CCPGPU_ERR_STATE, as
// ccpgpu_error_flags does for a handle; an escaped bead (clamped into the
// border cell of the grid) only sets its flag.
extern "C" int ccpgpu_noalloc_error_flags(int32_t *flags8, void *stream) {
  using namespace ccpgpu::noalloc;
  return guarded([&] {
    need(flags8 != nullptr, "null argument");
    int dev = 0;
    CK(cudaGetDevice(&dev));
    need(dev >= 0 && dev < MAX_DEVICES, "device index out of range");
    const int *err = reinterpret_cast<const int *>(scratch_base(dev) + OFF_ERR);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    CK(cudaMemcpyAsync(flags8, err, sizeof(int) * ERR_COUNT, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (flags8[ERR_NAN] || flags8[ERR_SLOT]) throw Error(ST_STATE, "device error flag set");
  });
}
