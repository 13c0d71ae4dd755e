// Host side of the contact-map surrogate (include/ccpgpu_surrogate.h): the
// layer launchers for the tcgen05 kernels, the network's forward and backward
// passes, AdamW, and the C ABI.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <random>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "../../include/ccpgpu.h"
#include "../../include/ccpgpu_surrogate.h"
#include "host.h"
#include "surrogate_kernels.cuh"

namespace sur {

using ccpgpu::Error;
using ccpgpu::ST_ARG;
using ccpgpu::ST_CUDA;
using ccpgpu::ST_PARAM;
using ccpgpu::ST_STATE;

#define SCK(x)                                                                     \
  do {                                                                             \
    cudaError_t e_ = (x);                                                          \
    if (e_ != cudaSuccess) throw Error(ST_CUDA, std::string("cuda: ") + cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
struct Buf {
  T *p = nullptr;
  size_t n = 0;
  Buf() = default;
  Buf(const Buf &) = delete;
  Buf &operator=(const Buf &) = delete;
  Buf(Buf &&o) noexcept : p(o.p), n(o.n) {
    o.p = nullptr;
    o.n = 0;
  }
  Buf &operator=(Buf &&o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      n = o.n;
      o.p = nullptr;
      o.n = 0;
    }
    return *this;
  }
  void alloc(size_t n_) {
    release();
    n = n_;
    if (n) SCK(cudaMalloc(&p, n * sizeof(T)));
  }
  void zero(cudaStream_t s) {
    if (n) SCK(cudaMemsetAsync(p, 0, n * sizeof(T), s));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  ~Buf() { release(); }
};

// ------------------------------------------------------------------ tensor maps

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                                  CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                  CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    SCK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !p) throw Error(ST_CUDA, "cuTensorMapEncodeTiled is unavailable");
    fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// Channels-last BF16 image [B][H][W][C] viewed as {C, W, H, B}; box {64, box_w, 1, 1}.
static CUtensorMap image_map(const void *ptr, int C, int W, int H, int B, int box_w) {
  CUtensorMap m;
  cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
  cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
  cuuint32_t box[4] = {64, (cuuint32_t)box_w, 1, 1};
  cuuint32_t es[4] = {1, 1, 1, 1};
  CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(ptr), dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(ST_CUDA, "image tensor map encoding failed");
  return m;
}

// Weights [rows][cin] BF16; box {64, box_rows}.
static CUtensorMap weight_map(const void *ptr, int cin, int rows, int box_rows) {
  CUtensorMap m;
  cuuint64_t dims[2] = {(cuuint64_t)cin, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)cin * 2};
  cuuint32_t box[2] = {64, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(ST_CUDA, "weight tensor map encoding failed");
  return m;
}

// ------------------------------------------------------------------ layer launchers

struct DevInfo {
  int sms = 0;
  int max_smem = 0;
};

static const DevInfo &dev_info() {
  static DevInfo d;
  static int dev_seen = -1;
  int dev = 0;
  SCK(cudaGetDevice(&dev));
  if (dev != dev_seen) {
    SCK(cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev));
    SCK(cudaDeviceGetAttribute(&d.max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    SCK(cudaFuncSetAttribute(k_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, d.max_smem));
    dev_seen = dev;
  }
  return d;
}

using Taps = std::vector<std::pair<int, int>>;  // (dh, dw)

static Taps negated(const Taps &t) {
  Taps r;
  for (auto &o : t) r.push_back({-o.first, -o.second});
  return r;
}

struct Launcher {
  cudaStream_t st = nullptr;
  int *err = nullptr;
  long long kernels = 0;

  // k_conv_tc over images of B x H x W pixels, cin -> N channels. The taps
  // must form an R x C grid with uniform steps (t = r C + c at ((r - R/2)
  // step_h, (c - C/2) step_w)), R in {1, 3}, C in {1, 3, 5}.
  void conv(const CUtensorMap &x, const CUtensorMap &w, int B, int H, int W, int cin, int N, const Taps &taps,
            const ConvEpi &epi) {
    const DevInfo &d = dev_info();
    if (W % 128 || (cin != 64 && cin != 128) || (N != 64 && N != 128))
      throw Error(ST_ARG, "convolution shape not supported (W % 128, channels 64 or 128)");
    const int nt = (int)taps.size();
    int R, C;
    if (nt == 9) R = 3, C = 3;
    else if (nt == 5) R = 1, C = 5;
    else if (nt == 3) R = 1, C = 3;
    else if (nt == 1) R = 1, C = 1;
    else throw Error(ST_ARG, "tap pattern not supported (3x3, 1x5, 1x3 or 1x1 grids)");
    ConvShape sh{};
    sh.B = B;
    sh.H = H;
    sh.W = W;
    sh.step_h = R > 1 ? taps[(R - 1) * C].first / (R / 2) : 0;
    sh.step_w = C > 1 ? taps[C - 1].second / (C / 2) : 0;
    for (int t = 0; t < nt; ++t)
      if (taps[t].first != (t / C - R / 2) * sh.step_h || taps[t].second != (t % C - C / 2) * sh.step_w)
        throw Error(ST_ARG, "tap pattern not supported (3x3, 1x5, 1x3 or 1x1 grids)");
    if (std::abs(sh.step_w) * (C / 2) > WIN_RADIUS) throw Error(ST_ARG, "tap column offset above the window radius");
    const int cb = cin / 64;
    sh.stages = MAX_STAGES;
    while (sh.stages > MMA_WARPS && (int)conv_smem_bytes(nt, cb, N, sh.stages) > d.max_smem)
      sh.stages -= MMA_WARPS;
    const uint32_t smem = conv_smem_bytes(nt, cb, N, sh.stages);
    if ((int)smem > d.max_smem) throw Error(ST_ARG, "convolution weights do not fit in shared memory");
    sh.n_tiles = B * H * (W / 128);
    if (sh.n_tiles == 0) return;
    const int grid = std::min(sh.n_tiles, d.sms);
    bool launched = false;
#define SUR_CONV(N_, R_, C_, CB_)                                                              \
  if (N == N_ && R == R_ && C == C_ && cb == CB_) {                                            \
    static bool attr = false;                                                                  \
    if (!attr) {                                                                               \
      SCK(cudaFuncSetAttribute(k_conv_tc<N_, R_, C_, CB_>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                               d.max_smem));                                                   \
      attr = true;                                                                             \
    }                                                                                          \
    k_conv_tc<N_, R_, C_, CB_><<<grid, CONV_THREADS, smem, st>>>(x, w, sh, epi, err);          \
    launched = true;                                                                           \
  }
#define SUR_CONV_N(R_, C_, CB_) SUR_CONV(64, R_, C_, CB_) SUR_CONV(128, R_, C_, CB_)
    SUR_CONV_N(3, 3, 1) SUR_CONV_N(3, 3, 2) SUR_CONV_N(1, 5, 1) SUR_CONV_N(1, 5, 2)
    SUR_CONV_N(1, 3, 1) SUR_CONV_N(1, 3, 2) SUR_CONV_N(1, 1, 1) SUR_CONV_N(1, 1, 2)
#undef SUR_CONV_N
#undef SUR_CONV
    if (!launched) throw Error(ST_ARG, "convolution configuration not instantiated");
    SCK(cudaGetLastError());
    ++kernels;
  }

  // Weight and bias gradients: dw [taps][N][cin], db [N] (may be null).
  // partial must hold partial_floats(...) floats.
  static void plan_wgrad(int B, int H, int W, int cin, int N, int ntaps, bool want_db, WgradShape &sh,
                         int &chunks, int &groups, uint32_t &smem) {
    const DevInfo &d = dev_info();
    if (W % 64 || cin % 64 || (N != 64 && N != 128)) throw Error(ST_ARG, "weight-gradient shape not supported");
    sh = WgradShape{};
    sh.B = B;
    sh.H = H;
    sh.W = W;
    sh.N = N;
    const int cbs = cin / 64;
    sh.n_x = ntaps * cbs;
    sh.n_atoms = sh.n_x + (want_db ? 1 : 0);
    if (sh.n_atoms & 1) ++sh.n_atoms;
    if (sh.n_atoms > MAX_ATOMS) throw Error(ST_ARG, "too many taps x channel blocks for the weight gradient");
    const int n_jobs = sh.n_atoms / 2;
    int jpg = std::min(n_jobs, 512 / N);
    while (jpg > 1 && (int)wgrad_smem_bytes(N, jpg) > d.max_smem) --jpg;
    smem = wgrad_smem_bytes(N, jpg);
    if ((int)smem > d.max_smem) throw Error(ST_ARG, "weight-gradient tiles do not fit in shared memory");
    sh.jobs_per_group = jpg;
    groups = (n_jobs + jpg - 1) / jpg;
    int cols = 32;
    while (cols < jpg * N) cols *= 2;
    sh.tmem_cols = cols;
    sh.kb_total = B * H * W / 64;
    const int want = std::max(1, d.sms / groups);
    sh.kb_per_cta = std::max(1, (sh.kb_total + want - 1) / want);
    chunks = (sh.kb_total + sh.kb_per_cta - 1) / sh.kb_per_cta;
  }

  static size_t partial_floats(int B, int H, int W, int cin, int N, int ntaps, bool want_db) {
    WgradShape sh;
    int chunks, groups;
    uint32_t smem;
    plan_wgrad(B, H, W, cin, N, ntaps, want_db, sh, chunks, groups, smem);
    return (size_t)chunks * sh.n_atoms * N * 64;
  }

  void wgrad(const CUtensorMap &x64, const CUtensorMap &y64, int B, int H, int W, int cin, int N, const Taps &taps,
             float *partial, size_t partial_cap, float *dw, float *db) {
    WgradShape sh;
    int chunks, groups;
    uint32_t smem;
    plan_wgrad(B, H, W, cin, N, (int)taps.size(), db != nullptr, sh, chunks, groups, smem);
    if (sh.kb_total == 0) return;
    const int cbs = cin / 64;
    for (int t = 0; t < (int)taps.size(); ++t)
      for (int c = 0; c < cbs; ++c) {
        const int a = t * cbs + c;
        sh.dh[a] = taps[t].first;
        sh.dw[a] = taps[t].second;
        sh.cb[a] = c;
      }
    if ((size_t)chunks * sh.n_atoms * N * 64 > partial_cap) throw Error(ST_STATE, "partial-sum buffer too small");
    k_wgrad_tc<<<dim3(chunks, groups), WG_THREADS, smem, st>>>(x64, y64, sh, partial, err);
    SCK(cudaGetLastError());
    k_wgrad_reduce<<<sh.n_x * N + (db ? N : 0), 256, 0, st>>>(partial, chunks, sh.n_atoms, sh.n_x, N, cbs, dw, db);
    SCK(cudaGetLastError());
    kernels += 2;
  }
};

static inline unsigned blocks(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// ------------------------------------------------------------------ network

struct Config {
  int seq_len = 1024, bins = 256, batch = 32;
  int enc_layers = 8, enc_width = 128, enc_kernel = 5;
  int head_layers = 6, head_width = 64;
  std::vector<int> dilations = {1, 2, 4, 8, 1, 2};
  float lr = 1e-3f, beta1 = 0.9f, beta2 = 0.999f, adam_eps = 1e-8f, weight_decay = 0.01f;
  float clip_norm = 1.0f;  // global gradient-norm clip before AdamW; 0: none
  long long lr_steps = 0;  // cosine decay of lr to lr_min over this many steps; 0: constant
  float lr_min = 0.0f;
};

static Config parse_config(const std::string &text) {
  ccpgpu::ParamMap pm(text);
  Config c;
  c.seq_len = pm.get<int>("seq_len", c.seq_len);
  c.bins = pm.get<int>("bins", c.bins);
  c.batch = pm.get<int>("batch", c.batch);
  c.enc_layers = pm.get<int>("enc_layers", c.enc_layers);
  c.enc_width = pm.get<int>("enc_width", c.enc_width);
  c.enc_kernel = pm.get<int>("enc_kernel", c.enc_kernel);
  c.head_layers = pm.get<int>("head_layers", c.head_layers);
  c.head_width = pm.get<int>("head_width", c.head_width);
  c.lr = pm.get<float>("lr", c.lr);
  c.beta1 = pm.get<float>("beta1", c.beta1);
  c.beta2 = pm.get<float>("beta2", c.beta2);
  c.adam_eps = pm.get<float>("adam_eps", c.adam_eps);
  c.weight_decay = pm.get<float>("weight_decay", c.weight_decay);
  c.clip_norm = pm.get<float>("clip_norm", c.clip_norm);
  c.lr_steps = (long long)pm.get<int>("lr_steps", 0);
  c.lr_min = pm.get<float>("lr_min", c.lr_min);
  if (pm.has("dilations")) {
    c.dilations.clear();
    std::string s = pm.raw("dilations");
    std::replace(s.begin(), s.end(), ',', ' ');
    std::istringstream is(s);
    int d;
    while (is >> d) c.dilations.push_back(d);
  } else {
    std::vector<int> def = c.dilations;
    c.dilations.clear();
    for (int l = 0; l < c.head_layers; ++l) c.dilations.push_back(def[l % def.size()]);
  }
  auto fail = [](const char *m) { throw Error(ST_PARAM, m); };
  if (c.seq_len < 128 || c.seq_len % 128) fail("seq_len must be a positive multiple of 128");
  if (c.bins < 128 || c.bins % 128 || c.seq_len % c.bins) fail("bins must be a multiple of 128 dividing seq_len");
  if (c.batch < 1 || c.batch > 4096) fail("batch out of range");
  if (c.enc_layers < 1 || c.enc_layers > 64) fail("enc_layers out of range");
  if (c.enc_width != 128) fail("enc_width must be 128");
  if (c.enc_kernel < 1 || c.enc_kernel > 5 || c.enc_kernel % 2 == 0) fail("enc_kernel must be 1, 3 or 5");
  if (c.head_layers < 1 || c.head_layers > 64) fail("head_layers out of range");
  if (c.head_width != 64) fail("head_width must be 64");
  if ((int)c.dilations.size() != c.head_layers) fail("dilations must list one value per head layer");
  for (int d : c.dilations)
    if (d < 1 || d > WIN_RADIUS) fail("dilation out of range");
  if (!(c.lr > 0)) fail("lr must be positive");
  if (!(c.clip_norm >= 0)) fail("clip_norm must be >= 0");
  if (c.lr_steps < 0 || !(c.lr_min >= 0) || c.lr_min > c.lr) fail("lr schedule out of range");
  return c;
}

struct Layer {
  int taps = 1, cin = 0, cout = 0;
  Taps off;
  size_t w_off = 0, b_off = 0;
  Buf<bf16> wb, wt;
  CUtensorMap map_w{}, map_wt{};
};

struct Net {
  Config cfg;
  int L, M, f;
  std::vector<Layer> enc, head;
  Layer proj;
  size_t E_off = 0, wo_off = 0, bo_off = 0, n_params = 0;
  struct Seg {
    size_t off, n;
    bool decay;
  };
  std::vector<Seg> segs;
  Buf<float> params, grads, adam_m, adam_v;
  long long step = 0;

  // activations (capacity cfg.batch)
  Buf<bf16> x0, hp, uv;
  std::vector<Buf<bf16>> h, z;             // h[1..enc_layers], z[0..head_layers]
  std::vector<Buf<uint32_t>> emask, hmask;  // emask[1..], hmask[1..]
  Buf<float> y, pred, dyb, dist_part;
  Buf<float> ps_dev;  // P(s) of one batch's predicted maps (predict_ps)
  Buf<uint8_t> decay;
  // backward
  Buf<float> hdz[2], edz[2], dhp;
  Buf<bf16> hdc[2], edc[2], duv;
  Buf<float> partial;
  Buf<double> loss, gsq;
  Buf<int> err;
  // tensor maps: *128 for the convolution (box of WIN_ROWS pixels: a tile of
  // 128 plus the tap margin), *64 for the weight gradient (box of 64 pixels)
  CUtensorMap m_x0_64{}, m_x0_128{}, m_hp_64{}, m_hp_128{}, m_duv_64{}, m_duv_128{};
  std::vector<CUtensorMap> m_h_64, m_h_128, m_z_64, m_z_128;
  CUtensorMap m_hdc_64[2]{}, m_hdc_128[2]{}, m_edc_64[2]{}, m_edc_128[2]{};
  // dataset
  Buf<uint8_t> ds_types, ds_lad;
  Buf<float> ds_target, ds_sweight;
  int ds_n = 0;
  Buf<int32_t> d_rows;
  Buf<uint8_t> in_types, in_lad;
  int32_t *h_rows = nullptr;  // pinned staging for row indices: two slots of `batch`
  cudaEvent_t ev_rows[2] = {nullptr, nullptr};
  int rows_slot = 0;
  // pinned staging of predicted maps: two slots of `batch` maps, drained into
  // the caller's buffer while the next batch runs
  float *h_maps = nullptr;
  cudaEvent_t ev_maps[2] = {nullptr, nullptr};
  float *pend_dst[2] = {nullptr, nullptr};
  size_t pend_n[2] = {0, 0};
  int maps_slot = 0;
  cudaStream_t st = nullptr;
  Launcher run;

  explicit Net(const Config &c, uint64_t seed) : cfg(c) {
    L = c.seq_len;
    M = c.bins;
    f = L / M;
    SCK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    run.st = st;
    // parameter layout
    size_t off = 0;
    auto conv_layer = [&](int taps, int cin, int cout, const Taps &o, bool decay) {
      Layer l;
      l.taps = taps;
      l.cin = cin;
      l.cout = cout;
      l.off = o;
      l.w_off = off;
      off += (size_t)taps * cout * cin;
      segs.push_back({l.w_off, (size_t)taps * cout * cin, decay});
      l.b_off = off;
      off += cout;
      segs.push_back({l.b_off, (size_t)cout, false});
      return l;
    };
    Taps enc_taps;
    for (int t = 0; t < c.enc_kernel; ++t) enc_taps.push_back({0, t - c.enc_kernel / 2});
    for (int l = 0; l < c.enc_layers; ++l) enc.push_back(conv_layer(c.enc_kernel, l == 0 ? 64 : 128, 128, enc_taps, true));
    proj = conv_layer(1, 128, 128, Taps{{0, 0}}, true);
    E_off = off;
    off += (size_t)M * 64;
    segs.push_back({E_off, (size_t)M * 64, false});
    for (int l = 0; l < c.head_layers; ++l) {
      const int d = c.dilations[l];
      Taps t;
      for (int a = -1; a <= 1; ++a)
        for (int b = -1; b <= 1; ++b) t.push_back({a * d, b * d});
      head.push_back(conv_layer(9, 64, 64, t, true));
    }
    wo_off = off;
    off += 64;
    segs.push_back({wo_off, 64, true});
    bo_off = off;
    off += 1;
    segs.push_back({bo_off, 1, false});
    n_params = off;

    params.alloc(n_params);
    grads.alloc(n_params);
    adam_m.alloc(n_params);
    adam_v.alloc(n_params);
    grads.zero(st);
    adam_m.zero(st);
    adam_v.zero(st);
    init_params(seed);
    {
      std::vector<uint8_t> dflag(n_params, 0);
      for (const Seg &sg : segs)
        if (sg.decay) std::fill(dflag.begin() + sg.off, dflag.begin() + sg.off + sg.n, (uint8_t)1);
      decay.alloc(n_params);
      SCK(cudaMemcpyAsync(decay.p, dflag.data(), n_params, cudaMemcpyHostToDevice, st));
      SCK(cudaStreamSynchronize(st));
    }
    for (Layer *l : all_layers()) {
      l->wb.alloc((size_t)l->taps * l->cout * l->cin);
      l->wt.alloc((size_t)l->taps * l->cout * l->cin);
      l->map_w = weight_map(l->wb.p, l->cin, l->taps * l->cout, l->cout);
      l->map_wt = weight_map(l->wt.p, l->cout, l->taps * l->cin, l->cin);
    }
    refresh_weights();
    alloc_activations();
    loss.alloc(1);
    gsq.alloc(1);
    err.alloc(1);
    err.zero(st);
    run.err = err.p;
    d_rows.alloc(c.batch);
    in_types.alloc((size_t)c.batch * L);
    in_lad.alloc((size_t)c.batch * L);
    SCK(cudaMallocHost(&h_rows, sizeof(int32_t) * 2 * c.batch));
    SCK(cudaMallocHost(&h_maps, sizeof(float) * 2 * (size_t)c.batch * M * M));
    for (int k = 0; k < 2; ++k) {
      SCK(cudaEventCreateWithFlags(&ev_rows[k], cudaEventDisableTiming));
      SCK(cudaEventCreateWithFlags(&ev_maps[k], cudaEventDisableTiming));
    }
    SCK(cudaStreamSynchronize(st));
  }

  ~Net() {
    if (st) cudaStreamSynchronize(st);
    if (h_rows) cudaFreeHost(h_rows);
    if (h_maps) cudaFreeHost(h_maps);
    for (int k = 0; k < 2; ++k) {
      if (ev_rows[k]) cudaEventDestroy(ev_rows[k]);
      if (ev_maps[k]) cudaEventDestroy(ev_maps[k]);
    }
    if (st) cudaStreamDestroy(st);
  }

  std::vector<Layer *> all_layers() {
    std::vector<Layer *> v;
    for (auto &l : enc) v.push_back(&l);
    v.push_back(&proj);
    for (auto &l : head) v.push_back(&l);
    return v;
  }

  void init_params(uint64_t seed) {
    std::vector<float> p(n_params, 0.0f);
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.0f, 1.0f);
    auto fill = [&](const Layer &l, float sd, int cin_real) {
      for (int t = 0; t < l.taps; ++t)
        for (int o = 0; o < l.cout; ++o)
          for (int i = 0; i < l.cin; ++i)
            p[l.w_off + ((size_t)t * l.cout + o) * l.cin + i] = i < cin_real ? sd * nd(rng) : 0.0f;
    };
    fill(enc[0], std::sqrt(2.0f / (3.0f * cfg.enc_kernel)), 3);
    for (int l = 1; l < cfg.enc_layers; ++l)
      fill(enc[l], std::sqrt(2.0f / (128.0f * cfg.enc_kernel)) / std::sqrt((float)cfg.enc_layers), 128);
    fill(proj, 1.0f / std::sqrt(128.0f), 128);
    for (int l = 0; l < cfg.head_layers; ++l)
      fill(head[l], std::sqrt(2.0f / (64.0f * 9.0f)) / std::sqrt((float)cfg.head_layers), 64);
    // output weights start at zero: the first prediction is the output bias
    // (the log of the dataset's mean contact probability) everywhere
    p[bo_off] = std::log(1e-3f);
    SCK(cudaMemcpyAsync(params.p, p.data(), n_params * sizeof(float), cudaMemcpyHostToDevice, st));
    SCK(cudaStreamSynchronize(st));
  }

  void refresh_weights() {
    WeightTable t{};
    long long most = 0;
    for (Layer *l : all_layers()) {
      if (t.n == MAX_LAYERS) throw Error(ST_PARAM, "too many layers");
      t.taps[t.n] = l->taps;
      t.co[t.n] = l->cout;
      t.ci[t.n] = l->cin;
      t.off[t.n] = (long long)l->w_off;
      t.wb[t.n] = l->wb.p;
      t.wt[t.n] = l->wt.p;
      most = std::max(most, (long long)l->taps * l->cout * l->cin);
      ++t.n;
    }
    k_weights_bf16<<<dim3(blocks(most), t.n), 256, 0, st>>>(params.p, t);
    SCK(cudaGetLastError());
    ++run.kernels;
  }

  void alloc_activations() {
    const int B = cfg.batch;
    const size_t PL = (size_t)B * L, PM = (size_t)B * M, PMM = (size_t)B * M * M;
    x0.alloc(PL * 64);
    m_x0_64 = image_map(x0.p, 64, L, 1, B, 64);
    m_x0_128 = image_map(x0.p, 64, L, 1, B, WIN_ROWS);
    h.resize(cfg.enc_layers + 1);
    emask.resize(cfg.enc_layers + 1);
    m_h_64.resize(cfg.enc_layers + 1);
    m_h_128.resize(cfg.enc_layers + 1);
    for (int l = 1; l <= cfg.enc_layers; ++l) {
      h[l].alloc(PL * 128);
      emask[l].alloc(PL * 4);
      m_h_64[l] = image_map(h[l].p, 128, L, 1, B, 64);
      m_h_128[l] = image_map(h[l].p, 128, L, 1, B, WIN_ROWS);
    }
    hp.alloc(PM * 128);
    uv.alloc(PM * 128);
    m_hp_64 = image_map(hp.p, 128, M, 1, B, 64);
    m_hp_128 = image_map(hp.p, 128, M, 1, B, WIN_ROWS);
    z.resize(cfg.head_layers + 1);
    hmask.resize(cfg.head_layers + 1);
    m_z_64.resize(cfg.head_layers + 1);
    m_z_128.resize(cfg.head_layers + 1);
    for (int l = 0; l <= cfg.head_layers; ++l) {
      z[l].alloc(PMM * 64);
      m_z_64[l] = image_map(z[l].p, 64, M, M, B, 64);
      m_z_128[l] = image_map(z[l].p, 64, M, M, B, WIN_ROWS);
      if (l > 0) hmask[l].alloc(PMM * 2);
    }
    y.alloc(PMM);
    pred.alloc(PMM);
    dyb.alloc(PMM);
    dist_part.alloc((size_t)B * M * 64);
    for (int k = 0; k < 2; ++k) {
      hdz[k].alloc(PMM * 64);
      hdc[k].alloc(PMM * 64);
      m_hdc_64[k] = image_map(hdc[k].p, 64, M, M, B, 64);
      m_hdc_128[k] = image_map(hdc[k].p, 64, M, M, B, WIN_ROWS);
      edz[k].alloc(PL * 128);
      edc[k].alloc(PL * 128);
      m_edc_64[k] = image_map(edc[k].p, 128, L, 1, B, 64);
      m_edc_128[k] = image_map(edc[k].p, 128, L, 1, B, WIN_ROWS);
    }
    duv.alloc(PM * 128);
    m_duv_64 = image_map(duv.p, 128, M, 1, B, 64);
    m_duv_128 = image_map(duv.p, 128, M, 1, B, WIN_ROWS);
    dhp.alloc(PM * 128);
    size_t pc = 0;
    pc = std::max(pc, Launcher::partial_floats(B, M, M, 64, 64, 9, true));
    pc = std::max(pc, Launcher::partial_floats(B, 1, M, 128, 128, 1, true));
    pc = std::max(pc, Launcher::partial_floats(B, 1, L, 128, 128, cfg.enc_kernel, true));
    pc = std::max(pc, Launcher::partial_floats(B, 1, L, 64, 128, cfg.enc_kernel, true));
    partial.alloc(pc);
  }

  // ---------------------------------------------------------------- passes

  // Forward over n sequences (types/lad device arrays, rows optional) into y;
  // `training` keeps what the backward pass needs (ReLU masks, last output).
  void forward(const uint8_t *types, const uint8_t *lad, const int32_t *rows, int n, bool training) {
    k_embed<<<blocks((long long)n * L), 256, 0, st>>>(types, lad, rows, L, n, x0.p);
    SCK(cudaGetLastError());
    ++run.kernels;
    for (int l = 0; l < cfg.enc_layers; ++l) {
      const Layer &ly = enc[l];
      ConvEpi e{};
      e.bias = params.p + ly.b_off;
      e.relu = 1;
      e.resid = l > 0 ? h[l].p : nullptr;
      e.out = h[l + 1].p;
      e.mask_out = training ? emask[l + 1].p : nullptr;
      run.conv(l == 0 ? m_x0_128 : m_h_128[l], ly.map_w, n, 1, L, ly.cin, 128, ly.off, e);
    }
    k_pool<<<blocks((long long)n * M * 128), 256, 0, st>>>(h[cfg.enc_layers].p, L, 128, f, n, hp.p);
    SCK(cudaGetLastError());
    ++run.kernels;
    {
      ConvEpi e{};
      e.bias = params.p + proj.b_off;
      e.out = uv.p;
      run.conv(m_hp_128, proj.map_w, n, 1, M, 128, 128, proj.off, e);
    }
    k_pair_fwd<<<dim3(M / PAIR_ROWS, n), 256, 0, st>>>(uv.p, params.p + E_off, M, z[0].p);
    SCK(cudaGetLastError());
    ++run.kernels;
    const long long P = (long long)n * M * M;
    SCK(cudaMemsetAsync(y.p, 0, sizeof(float) * P, st));
    for (int l = 0; l < cfg.head_layers; ++l) {
      const Layer &ly = head[l];
      const bool last = l == cfg.head_layers - 1;
      ConvEpi e{};
      e.bias = params.p + ly.b_off;
      e.relu = 1;
      e.resid = z[l].p;
      // the last layer's output is needed only by the backward pass
      e.out = (!last || training) ? z[l + 1].p : nullptr;
      e.mask_out = training ? hmask[l + 1].p : nullptr;
      if (last) {  // output layer fused into the epilogue
        e.wo = params.p + wo_off;
        e.bo = params.p + bo_off;
        e.y = y.p;
      }
      run.conv(m_z_128[l], ly.map_w, n, M, M, 64, 64, ly.off, e);
    }
  }

  // Backward of the loss on dataset rows (after forward on the same rows).
  void backward(const int32_t *rows, int n) {
    SCK(cudaMemsetAsync(grads.p + wo_off, 0, 65 * sizeof(float), st));
    SCK(cudaMemsetAsync(loss.p, 0, sizeof(double), st));
    const long long P = (long long)n * M * M;
    const int HL = cfg.head_layers;
    k_loss_out_bwd<<<blocks(P), 256, 0, st>>>(y.p, ds_target.p, ds_sweight.p, rows, z[HL].p, hmask[HL].p,
                                              params.p + wo_off, M, n, dyb.p, hdc[0].p, grads.p + wo_off,
                                              grads.p + bo_off, loss.p);
    SCK(cudaGetLastError());
    ++run.kernels;
    int kc = 0;   // dc_l is in hdc[kc]
    int kz = -1;  // dz_{l+1} is in hdz[kz]; -1: the rank-1 dy wo of the output layer
    for (int l = HL - 1; l >= 0; --l) {
      const Layer &ly = head[l];
      run.wgrad(m_z_64[l], m_hdc_64[kc], n, M, M, 64, 64, ly.off, partial.p, partial.n, grads.p + ly.w_off,
                grads.p + ly.b_off);
      ConvEpi e{};
      if (kz >= 0) {
        e.resid_f32 = hdz[kz].p;
      } else {
        e.resid_dy = dyb.p;
        e.wo = params.p + wo_off;
      }
      const int oz = kz == 0 ? 1 : 0;
      e.out_f32 = hdz[oz].p;
      if (l > 0) {
        e.mask_in = hmask[l].p;
        e.out = hdc[kc ^ 1].p;
      }
      run.conv(m_hdc_128[kc], ly.map_wt, n, M, M, 64, 64, negated(ly.off), e);
      kz = oz;
      kc ^= 1;
    }
    const int k = kz;  // dz0
    k_pair_bwd<<<dim3(M, n), 256, 0, st>>>(hdz[k].p, uv.p, M, duv.p);
    k_dist_bwd<<<dim3(M, n), 256, 0, st>>>(hdz[k].p, M, dist_part.p);
    k_dist_reduce<<<blocks((long long)M * 64), 256, 0, st>>>(dist_part.p, M, n, grads.p + E_off);
    SCK(cudaGetLastError());
    run.kernels += 3;
    run.wgrad(m_hp_64, m_duv_64, n, 1, M, 128, 128, proj.off, partial.p, partial.n, grads.p + proj.w_off,
              grads.p + proj.b_off);
    {
      ConvEpi e{};
      e.out_f32 = dhp.p;
      run.conv(m_duv_128, proj.map_wt, n, 1, M, 128, 128, proj.off, e);
    }
    const int EL = cfg.enc_layers;
    k_unpool<<<blocks((long long)n * L * 8), 256, 0, st>>>(dhp.p, emask[EL].p, L, f, n, edz[0].p, edc[0].p);
    SCK(cudaGetLastError());
    ++run.kernels;
    int ke = 0;
    for (int l = EL - 1; l >= 1; --l) {
      const Layer &ly = enc[l];
      run.wgrad(m_h_64[l], m_edc_64[ke], n, 1, L, 128, 128, ly.off, partial.p, partial.n, grads.p + ly.w_off,
                grads.p + ly.b_off);
      ConvEpi e{};
      e.resid_f32 = edz[ke].p;
      e.out_f32 = edz[ke ^ 1].p;
      e.mask_in = emask[l].p;
      e.out = edc[ke ^ 1].p;
      run.conv(m_edc_128[ke], ly.map_wt, n, 1, L, 128, 128, negated(ly.off), e);
      ke ^= 1;
    }
    run.wgrad(m_x0_64, m_edc_64[ke], n, 1, L, 64, 128, enc[0].off, partial.p, partial.n, grads.p + enc[0].w_off,
              grads.p + enc[0].b_off);
  }

  void adamw() {
    ++step;
    const float bc1 = 1.0f - std::pow(cfg.beta1, (float)step);
    const float bc2 = 1.0f - std::pow(cfg.beta2, (float)step);
    float lr = cfg.lr;
    if (cfg.lr_steps > 0) {
      const double f = std::min(1.0, (double)(step - 1) / (double)cfg.lr_steps);
      lr = (float)(cfg.lr_min + 0.5 * (cfg.lr - cfg.lr_min) * (1.0 + std::cos(3.14159265358979323846 * f)));
    }
    SCK(cudaMemsetAsync(gsq.p, 0, sizeof(double), st));
    k_grad_sq<<<std::min<long long>(blocks((long long)n_params), 1024), 256, 0, st>>>(grads.p, (long long)n_params,
                                                                                       gsq.p);
    k_adamw<<<blocks((long long)n_params), 256, 0, st>>>(params.p, grads.p, adam_m.p, adam_v.p, decay.p,
                                                         (long long)n_params, lr, cfg.beta1, cfg.beta2,
                                                         cfg.adam_eps, cfg.weight_decay, bc1, bc2, cfg.clip_norm,
                                                         gsq.p);
    SCK(cudaGetLastError());
    run.kernels += 2;
    refresh_weights();
  }

  const int32_t *upload_rows(const int32_t *rows, int n) {
    if (n < 1 || n > cfg.batch) throw Error(ST_ARG, "row count must be in [1, batch]");
    if (ds_n == 0) throw Error(ST_STATE, "no dataset");
    // alternate pinned slots; wait only for the copy that last read this slot
    rows_slot ^= 1;
    int32_t *hr = h_rows + (size_t)rows_slot * cfg.batch;
    SCK(cudaEventSynchronize(ev_rows[rows_slot]));
    for (int i = 0; i < n; ++i) {
      if (rows[i] < 0 || rows[i] >= ds_n) throw Error(ST_ARG, "dataset row out of range");
      hr[i] = rows[i];
    }
    SCK(cudaMemcpyAsync(d_rows.p, hr, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
    SCK(cudaEventRecord(ev_rows[rows_slot], st));
    return d_rows.p;
  }

  void check_flags() {
    int flags = 0;
    SCK(cudaMemcpyAsync(&flags, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    SCK(cudaStreamSynchronize(st));
    if (flags) {
      err.zero(st);
      throw Error(ST_STATE, std::string("a tensor-core kernel (") +
                                ((flags & 1) ? "convolution" : "") +
                                ((flags & 3) == 3 ? ", " : "") +
                                ((flags & 2) ? "weight gradient" : "") +
                                ") gave up waiting for its pipeline");
    }
  }

  double loss_grad(const int32_t *rows_host, int n, bool update, bool want_loss) {
    const int32_t *rows = upload_rows(rows_host, n);
    forward(ds_types.p, ds_lad.p, rows, n, true);
    backward(rows, n);
    if (update) adamw();
    double l = 0;
    if (want_loss) {
      SCK(cudaMemcpyAsync(&l, loss.p, sizeof(double), cudaMemcpyDeviceToHost, st));
      check_flags();
    }
    return l;
  }

  // Maps of the last forward pass: to the device buffer `pred`, and with
  // maps_host through a pinned slot into maps_host[first ...]; the slot is
  // copied out by drain_maps while later batches run.
  void predict_out(int n, float *maps_host, size_t first) {
    const long long P = (long long)n * M * M;
    k_predict_maps<<<blocks(P), 256, 0, st>>>(y.p, M, n, pred.p);
    SCK(cudaGetLastError());
    ++run.kernels;
    if (!maps_host) return;
    maps_slot ^= 1;
    drain_slot(maps_slot);
    float *stage = h_maps + (size_t)maps_slot * cfg.batch * M * M;
    SCK(cudaMemcpyAsync(stage, pred.p, sizeof(float) * P, cudaMemcpyDeviceToHost, st));
    SCK(cudaEventRecord(ev_maps[maps_slot], st));
    pend_dst[maps_slot] = maps_host + first * (size_t)M * M;
    pend_n[maps_slot] = (size_t)P;
    drain_slot(maps_slot ^ 1);
  }

  void drain_slot(int k) {
    if (!pend_dst[k]) return;
    SCK(cudaEventSynchronize(ev_maps[k]));
    std::memcpy(pend_dst[k], h_maps + (size_t)k * cfg.batch * M * M, sizeof(float) * pend_n[k]);
    pend_dst[k] = nullptr;
  }

  // forget copies owed to an earlier call that failed part-way
  void discard_pending() { pend_dst[0] = pend_dst[1] = nullptr; }

  void drain_maps() {
    drain_slot(maps_slot ^ 1);
    drain_slot(maps_slot);
  }
};

}  // namespace sur

using namespace sur;

struct ccpsur_net {
  std::unique_ptr<Net> n;
};

template <typename F>
static int sguard(F &&f) {
  try {
    f();
    return CCPGPU_OK;
  } catch (const Error &e) {
    ccpgpu::set_last_error(e.what());
    return e.code;
  } catch (const std::bad_alloc &) {
    ccpgpu::set_last_error("out of host memory");
    return CCPGPU_ERR_ARG;
  } catch (const std::exception &e) {
    ccpgpu::set_last_error(e.what());
    return CCPGPU_ERR_ARG;
  }
}

static void sneed(bool c, const char *m) {
  if (!c) throw Error(ST_ARG, m);
}

static Net &net_of(ccpsur_net *h) {
  sneed(h && h->n, "null handle");
  return *h->n;
}

extern "C" {

int ccpsur_create(const char *config_text, uint64_t seed, ccpsur_net **out) {
  return sguard([&] {
    sneed(config_text && out, "null argument");
    *out = nullptr;
    Config c = parse_config(config_text);
    auto h = std::make_unique<ccpsur_net>();
    h->n = std::make_unique<Net>(c, seed);
    *out = h.release();
  });
}

int ccpsur_destroy(ccpsur_net *h) {
  return sguard([&] { delete h; });
}

int ccpsur_info_get(const ccpsur_net *h, ccpsur_info *out) {
  return sguard([&] {
    sneed(h && h->n && out, "null argument");
    const Net &n = *h->n;
    out->seq_len = n.cfg.seq_len;
    out->bins = n.cfg.bins;
    out->batch = n.cfg.batch;
    out->enc_layers = n.cfg.enc_layers;
    out->enc_width = n.cfg.enc_width;
    out->enc_kernel = n.cfg.enc_kernel;
    out->head_layers = n.cfg.head_layers;
    out->head_width = n.cfg.head_width;
    out->dataset_size = n.ds_n;
    out->n_params = (int64_t)n.n_params;
    out->step = n.step;
  });
}

int ccpsur_get_params(ccpsur_net *h, float *out, int64_t cnt) {
  return sguard([&] {
    Net &n = net_of(h);
    sneed(out && cnt == (int64_t)n.n_params, "parameter count mismatch");
    SCK(cudaMemcpyAsync(out, n.params.p, sizeof(float) * cnt, cudaMemcpyDeviceToHost, n.st));
    SCK(cudaStreamSynchronize(n.st));
  });
}

int ccpsur_set_params(ccpsur_net *h, const float *in, int64_t cnt) {
  return sguard([&] {
    Net &n = net_of(h);
    sneed(in && cnt == (int64_t)n.n_params, "parameter count mismatch");
    SCK(cudaMemcpyAsync(n.params.p, in, sizeof(float) * cnt, cudaMemcpyHostToDevice, n.st));
    n.refresh_weights();
    SCK(cudaStreamSynchronize(n.st));
  });
}

int ccpsur_get_grads(ccpsur_net *h, float *out, int64_t cnt) {
  return sguard([&] {
    Net &n = net_of(h);
    sneed(out && cnt == (int64_t)n.n_params, "parameter count mismatch");
    SCK(cudaMemcpyAsync(out, n.grads.p, sizeof(float) * cnt, cudaMemcpyDeviceToHost, n.st));
    SCK(cudaStreamSynchronize(n.st));
  });
}

int ccpsur_set_dataset(ccpsur_net *h, const uint8_t *types, const uint8_t *lad, const float *maps, int32_t cnt) {
  return sguard([&] {
    Net &n = net_of(h);
    sneed(types && maps && cnt > 0, "null argument or empty dataset");
    const size_t L = n.L, M = n.M, MM = M * M;
    for (size_t k = 0; k < (size_t)cnt * L; ++k) sneed(types[k] <= 1, "bead type must be 0 (A) or 1 (B)");
    double total = 0;
    std::vector<double> ps(M, 0.0);
    for (size_t k = 0; k < (size_t)cnt * MM; ++k) {
      sneed(std::isfinite(maps[k]) && maps[k] >= 0.0f && maps[k] <= 1.0f,
            "contact probabilities must be finite and in [0, 1]");
      const size_t r = k % MM, i = r / M, j = r % M;
      ps[i > j ? i - j : j - i] += maps[k];
      total += maps[k];
    }
    // separation weights: w[s] = M / (mean P(s) x bin pairs at separation s),
    // so every separation carries the same total weight (relative to its
    // contact probability); the mean over all pixels of w[s] P(s) is 1
    std::vector<float> sw(M);
    for (size_t s = 0; s < M; ++s) {
      const double npairs = (double)(s == 0 ? M : 2 * (M - s));
      sw[s] = (float)((double)M / (std::max(ps[s] / ((double)cnt * npairs), 1e-6) * npairs));
    }
    std::vector<uint8_t> lf((size_t)cnt * L, 0);
    if (lad)
      for (size_t k = 0; k < lf.size(); ++k) lf[k] = lad[k] ? 1 : 0;
    n.ds_types.alloc((size_t)cnt * L);
    n.ds_lad.alloc((size_t)cnt * L);
    n.ds_target.alloc((size_t)cnt * MM);
    n.ds_sweight.alloc(M);
    SCK(cudaMemcpyAsync(n.ds_types.p, types, (size_t)cnt * L, cudaMemcpyHostToDevice, n.st));
    SCK(cudaMemcpyAsync(n.ds_lad.p, lf.data(), lf.size(), cudaMemcpyHostToDevice, n.st));
    SCK(cudaMemcpyAsync(n.ds_target.p, maps, sizeof(float) * (size_t)cnt * MM, cudaMemcpyHostToDevice, n.st));
    SCK(cudaMemcpyAsync(n.ds_sweight.p, sw.data(), sizeof(float) * M, cudaMemcpyHostToDevice, n.st));
    n.ds_n = cnt;
    if (n.step == 0) {  // start the output bias at the log of the mean contact probability
      const float bo = (float)std::log(std::max(total / ((double)cnt * MM), 1e-6));
      SCK(cudaMemcpyAsync(n.params.p + n.bo_off, &bo, sizeof(float), cudaMemcpyHostToDevice, n.st));
    }
    SCK(cudaStreamSynchronize(n.st));
  });
}

int ccpsur_loss_grad(ccpsur_net *h, const int32_t *rows, int32_t cnt, double *loss) {
  return sguard([&] {
    Net &n = net_of(h);
    sneed(rows, "null argument");
    double l = n.loss_grad(rows, cnt, false, true);
    if (loss) *loss = l;
  });
}

int ccpsur_train_step(ccpsur_net *h, const int32_t *rows, int32_t cnt, double *loss) {
  return sguard([&] {
    Net &n = net_of(h);
    sneed(rows, "null argument");
    double l = n.loss_grad(rows, cnt, true, loss != nullptr);
    if (loss) *loss = l;
  });
}

int ccpsur_predict(ccpsur_net *h, const uint8_t *types, const uint8_t *lad, int32_t cnt, float *maps) {
  return sguard([&] {
    Net &n = net_of(h);
    sneed(types && maps && cnt >= 0, "null argument");
    const size_t L = n.L;
    n.discard_pending();
    for (int32_t first = 0; first < cnt; first += n.cfg.batch) {
      const int b = std::min(n.cfg.batch, cnt - first);
      // pageable sources: the copies return once the data is staged
      SCK(cudaMemcpyAsync(n.in_types.p, types + (size_t)first * L, (size_t)b * L, cudaMemcpyHostToDevice, n.st));
      if (lad)
        SCK(cudaMemcpyAsync(n.in_lad.p, lad + (size_t)first * L, (size_t)b * L, cudaMemcpyHostToDevice, n.st));
      n.forward(n.in_types.p, lad ? n.in_lad.p : nullptr, nullptr, b, false);
      n.predict_out(b, maps, first);
    }
    n.drain_maps();
    n.check_flags();
  });
}

int ccpsur_predict_ps(ccpsur_net *h, const uint8_t *types, const uint8_t *lad, int32_t cnt,
                      float *ps) {
  return sguard([&] {
    Net &n = net_of(h);
    sneed(types && ps && cnt >= 0, "null argument");
    const size_t L = n.L;
    const int M = n.M;
    if (n.ps_dev.n < (size_t)n.cfg.batch * M) n.ps_dev.alloc((size_t)n.cfg.batch * M);
    n.discard_pending();
    for (int32_t first = 0; first < cnt; first += n.cfg.batch) {
      const int b = std::min(n.cfg.batch, cnt - first);
      SCK(cudaMemcpyAsync(n.in_types.p, types + (size_t)first * L, (size_t)b * L, cudaMemcpyHostToDevice, n.st));
      if (lad)
        SCK(cudaMemcpyAsync(n.in_lad.p, lad + (size_t)first * L, (size_t)b * L, cudaMemcpyHostToDevice, n.st));
      n.forward(n.in_types.p, lad ? n.in_lad.p : nullptr, nullptr, b, false);
      n.predict_out(b, nullptr, first);
      k_ps_curve<<<b, 256, 0, n.st>>>(n.pred.p, M, n.ps_dev.p);
      SCK(cudaGetLastError());
      ++n.run.kernels;
      SCK(cudaMemcpyAsync(ps + (size_t)first * M, n.ps_dev.p, sizeof(float) * (size_t)b * M,
                          cudaMemcpyDeviceToHost, n.st));
    }
    n.check_flags();
  });
}

int ccpsur_predict_rows(ccpsur_net *h, const int32_t *rows, int32_t cnt, float *maps) {
  return sguard([&] {
    Net &n = net_of(h);
    sneed(rows && cnt >= 0, "null argument");
    n.discard_pending();
    for (int32_t first = 0; first < cnt; first += n.cfg.batch) {
      const int b = std::min(n.cfg.batch, cnt - first);
      const int32_t *r = n.upload_rows(rows + first, b);
      n.forward(n.ds_types.p, n.ds_lad.p, r, b, false);
      n.predict_out(b, maps, first);
    }
    if (maps) {
      n.drain_maps();
      n.check_flags();
    }
  });
}

int ccpsur_synchronize(ccpsur_net *h) {
  return sguard([&] {
    Net &n = net_of(h);
    n.check_flags();
  });
}

int ccpsur_stream_handle(ccpsur_net *h, void **stream) {
  return sguard([&] {
    Net &n = net_of(h);
    sneed(stream, "null argument");
    *stream = (void *)n.st;
  });
}

int ccpsur_error_flags(ccpsur_net *h, int32_t *flags) {
  return sguard([&] {
    Net &n = net_of(h);
    sneed(flags, "null argument");
    int f = 0;
    SCK(cudaMemcpyAsync(&f, n.err.p, sizeof(int), cudaMemcpyDeviceToHost, n.st));
    SCK(cudaStreamSynchronize(n.st));
    n.err.zero(n.st);
    *flags = f;
  });
}

int ccpsur_kernel_count(const ccpsur_net *h, int64_t *cnt) {
  return sguard([&] {
    sneed(h && h->n && cnt, "null argument");
    *cnt = h->n->run.kernels;
  });
}

static Taps taps_of(int32_t ntaps, const int32_t *dh, const int32_t *dw) {
  sneed(ntaps >= 1 && ntaps <= MAX_TAPS && dh && dw, "taps out of range");
  Taps t;
  for (int i = 0; i < ntaps; ++i) t.push_back({dh[i], dw[i]});
  return t;
}

int ccpsur_conv_bf16(int32_t B, int32_t H, int32_t W, int32_t cin, int32_t cout, int32_t ntaps, const int32_t *dh,
                     const int32_t *dw, const uint16_t *x, const uint16_t *w, const float *bias, int32_t relu,
                     const uint16_t *resid, uint16_t *out, uint32_t *mask_out) {
  return sguard([&] {
    sneed(B > 0 && H > 0 && W > 0 && x && w && out, "null argument or empty image");
    sneed((cin == 64 || cin == 128) && (cout == 64 || cout == 128), "channels must be 64 or 128");
    Taps taps = taps_of(ntaps, dh, dw);
    const size_t P = (size_t)B * H * W;
    cudaStream_t st;
    SCK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard {
      cudaStream_t s;
      ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{st};
    Buf<bf16> dx, dwb, dres, dout;
    Buf<float> dbias;
    Buf<uint32_t> dmask;
    Buf<int> derr;
    dx.alloc(P * cin);
    dwb.alloc((size_t)ntaps * cout * cin);
    dout.alloc(P * cout);
    derr.alloc(1);
    derr.zero(st);
    SCK(cudaMemcpyAsync(dx.p, x, P * cin * 2, cudaMemcpyHostToDevice, st));
    SCK(cudaMemcpyAsync(dwb.p, w, (size_t)ntaps * cout * cin * 2, cudaMemcpyHostToDevice, st));
    ConvEpi e{};
    if (bias) {
      dbias.alloc(cout);
      SCK(cudaMemcpyAsync(dbias.p, bias, cout * 4, cudaMemcpyHostToDevice, st));
      e.bias = dbias.p;
    }
    if (resid) {
      dres.alloc(P * cout);
      SCK(cudaMemcpyAsync(dres.p, resid, P * cout * 2, cudaMemcpyHostToDevice, st));
      e.resid = dres.p;
    }
    if (mask_out) {
      dmask.alloc(P * cout / 32);
      e.mask_out = dmask.p;
    }
    e.relu = relu ? 1 : 0;
    e.out = dout.p;
    Launcher run;
    run.st = st;
    run.err = derr.p;
    CUtensorMap mx = image_map(dx.p, cin, W, H, B, WIN_ROWS);
    CUtensorMap mw = weight_map(dwb.p, cin, ntaps * cout, cout);
    run.conv(mx, mw, B, H, W, cin, cout, taps, e);
    int flags = 0;
    SCK(cudaMemcpyAsync(out, dout.p, P * cout * 2, cudaMemcpyDeviceToHost, st));
    if (mask_out) SCK(cudaMemcpyAsync(mask_out, dmask.p, P * cout / 32 * 4, cudaMemcpyDeviceToHost, st));
    SCK(cudaMemcpyAsync(&flags, derr.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    SCK(cudaStreamSynchronize(st));
    if (flags) throw Error(ST_STATE, "the convolution kernel gave up waiting for its pipeline");
  });
}

int ccpsur_wgrad_bf16(int32_t B, int32_t H, int32_t W, int32_t cin, int32_t cout, int32_t ntaps, const int32_t *dh,
                      const int32_t *dw, const uint16_t *x, const uint16_t *dy, float *dw_out, float *db_out) {
  return sguard([&] {
    sneed(B > 0 && H > 0 && W > 0 && x && dy && dw_out, "null argument or empty image");
    sneed((cin == 64 || cin == 128) && (cout == 64 || cout == 128), "channels must be 64 or 128");
    Taps taps = taps_of(ntaps, dh, dw);
    const size_t P = (size_t)B * H * W;
    cudaStream_t st;
    SCK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard {
      cudaStream_t s;
      ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{st};
    Buf<bf16> dx, ddy;
    Buf<float> dwo, dbo, part;
    Buf<int> derr;
    dx.alloc(P * cin);
    ddy.alloc(P * cout);
    dwo.alloc((size_t)ntaps * cout * cin);
    if (db_out) dbo.alloc(cout);
    derr.alloc(1);
    derr.zero(st);
    part.alloc(Launcher::partial_floats(B, H, W, cin, cout, ntaps, db_out != nullptr));
    SCK(cudaMemcpyAsync(dx.p, x, P * cin * 2, cudaMemcpyHostToDevice, st));
    SCK(cudaMemcpyAsync(ddy.p, dy, P * cout * 2, cudaMemcpyHostToDevice, st));
    Launcher run;
    run.st = st;
    run.err = derr.p;
    CUtensorMap mx = image_map(dx.p, cin, W, H, B, 64);
    CUtensorMap my = image_map(ddy.p, cout, W, H, B, 64);
    run.wgrad(mx, my, B, H, W, cin, cout, taps, part.p, part.n, dwo.p, db_out ? dbo.p : nullptr);
    int flags = 0;
    SCK(cudaMemcpyAsync(dw_out, dwo.p, (size_t)ntaps * cout * cin * 4, cudaMemcpyDeviceToHost, st));
    if (db_out) SCK(cudaMemcpyAsync(db_out, dbo.p, cout * 4, cudaMemcpyDeviceToHost, st));
    SCK(cudaMemcpyAsync(&flags, derr.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    SCK(cudaStreamSynchronize(st));
    if (flags) throw Error(ST_STATE, "the weight-gradient kernel gave up waiting for its pipeline");
  });
}

}  // extern "C"
