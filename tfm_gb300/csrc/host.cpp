// Host-side pieces: ccp parameter map and range checks, force-field presets,
// initial-condition generator and ccp file formats.
#include "host.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <limits>
#include <sstream>
#include <unordered_map>

namespace ccpgpu {

// ------------------------------------------------------------ parameter map

ParamMap::ParamMap(const std::string &text) {
  std::istringstream is(text);
  std::string k, v;
  while (is >> k >> v) {
    if (!has(k)) kv.emplace_back(k, v);  // std::map::insert keeps the first value
  }
}

bool ParamMap::has(const std::string &k) const {
  for (auto &p : kv)
    if (p.first == k) return true;
  return false;
}

std::string ParamMap::raw(const std::string &k) const {
  for (auto &p : kv)
    if (p.first == k) return p.second;
  return std::string();
}

template <typename T>
T ParamMap::get(const std::string &k, T def) const {
  if (!has(k)) return def;
  T val{};
  std::stringstream{raw(k)} >> val;
  return val;
}
template uint32_t ParamMap::get<uint32_t>(const std::string &, uint32_t) const;
template int ParamMap::get<int>(const std::string &, int) const;
template float ParamMap::get<float>(const std::string &, float) const;
template double ParamMap::get<double>(const std::string &, double) const;
template uint64_t ParamMap::get<uint64_t>(const std::string &, uint64_t) const;
template std::string ParamMap::get<std::string>(const std::string &, std::string) const;

static void fail(const std::string &m) { throw Error(ST_PARAM, m); }

Geometry make_geometry(float R_n, float R_o, float R_b) {
  Geometry g;
  g.R_n = R_n;
  g.R_o = R_o;
  g.R_b = R_b;
  g.noc = std::cos(std::asin(R_o / R_n));
  g.boc = std::cos(std::asin(R_o / R_b));
  g.nod = std::sqrt(R_n * R_n - R_o * R_o);
  g.bod = std::sqrt(R_b * R_b - R_o * R_o);
  g.d_b = g.nod + g.bod;
  g.d_m = g.d_b + R_b;
  return g;
}

static ForceField preset_ccp(float T) {
  ForceField f{};
  f.pot = POT_WF;
  f.bend_all = 0;
  f.k_e = 128.0f;
  f.l_0 = 1.0f;
  f.k_b = 1.0f;
  f.e_att = 0.5f;
  f.e_rep = 0.5f;
  f.rc_rep = CCP_RCO;
  f.rc_att = CCP_ACO;
  f.e_w = 1.0f;
  f.rc_w = CCP_RCO;
  f.e_l = 8.0f;
  f.lco = CCP_LCO;
  f.lbs_depth = CCP_RCO;
  f.k_icg = 128.0f;
  f.rc_icg = CCP_RCO;
  f.mis = CCP_MIS;
  f.max_step = 0.0f;
  // ccp's relaxation has no cap either (chrsim.cu:500-509), but there a bead
  // pushed within ~0.35 sigma of the wall by overlapping neighbours gets a
  // Wang-Frenkel wall force (~96 / gap^7) that moves it hundreds of sigma in
  // one step, out of the nucleus; 16 relaxations of 30385-bead walks never
  // finished without one. The soft repulsion alone moves a bead < 0.07 sigma
  // per overlapping neighbour and stage, so a 0.25 sigma cap leaves ordinary
  // relaxation steps as they are.
  f.icg_max_step = 0.25f;
  f.dt = (float)CCP_DT;
  f.kT = CCP_K_B * T;
  f.sd = (float)std::sqrt(2.0 * CCP_K_B * T * CCP_DT);  // chrsim.cu:424
  return f;
}

static ForceField preset_baseline(float kT, float dt) {
  ForceField f{};
  const float wca = std::pow(2.0f, 1.0f / 6.0f);
  f.pot = POT_LJ;
  f.bend_all = 1;
  f.k_e = 100.0f;
  f.l_0 = 1.0f;
  f.k_b = 2.0f;
  f.e_att = 0.5f;
  f.e_rep = 1.0f;
  f.rc_rep = wca;
  f.rc_att = 2.5f;
  f.e_w = 1.0f;
  f.rc_w = wca;
  f.e_l = 8.0f;
  f.lco = CCP_LCO;
  f.lbs_depth = wca;
  f.k_icg = 128.0f;
  f.rc_icg = CCP_RCO;
  // WCA with dt = 1e-3 is stable (dt |dF/dr| < 2) only beyond r ~ 0.92
  f.mis = 0.95f;
  // a 5-sigma noise jump can bring a WCA pair to r ~ 0.7, where one corrector
  // step would move it several sigma: cap the deterministic displacement
  f.max_step = 0.1f;
  f.icg_max_step = f.max_step;
  f.dt = dt;
  f.kT = kT;
  f.sd = (float)std::sqrt(2.0 * (double)kT * (double)dt);
  return f;
}

ForceField make_preset(int preset) {
  return preset == PRESET_CCP ? preset_ccp(298.0f) : preset_baseline(1.0f, 1.0e-3f);
}

Params parse_params(const std::string &text) {
  ParamMap pm(text);
  Params p;
  std::string ffs = pm.get<std::string>("force_field", "ccp");
  if (ffs == "ccp")
    p.preset = PRESET_CCP;
  else if (ffs == "baseline")
    p.preset = PRESET_BASELINE;
  else
    fail("force_field out of range");
  p.relaxed = pm.get<int>("relaxed_limits", p.preset == PRESET_BASELINE ? 1 : 0) != 0;

  // nucleus geometry (cngeom, chrdat.cu:13-30)
  if (p.preset == PRESET_CCP) {
    p.N = pm.get<uint32_t>("number_of_particles", CCP_N_DEF);
    p.R_n = pm.get<float>("nucleus_radius", 0.0f);
  } else {
    p.N = pm.get<uint32_t>("number_of_particles", 2048u);
    p.packing_fraction = pm.get<float>("packing_fraction", 0.2f);
    p.R_n = pm.get<float>("nucleus_radius",
                          (float)(0.5 * std::cbrt((double)p.N / p.packing_fraction)));
  }
  p.R_o = pm.get<float>("opening_radius", 0.0f);
  p.R_b = pm.get<float>("bleb_radius", 0.0f);
  const float r_max = p.relaxed ? 1.0e4f : 100.0f;
  if (!(0.0f < p.R_n && p.R_n < r_max)) fail("nucleus_radius out of range");
  if (!(0.0f <= p.R_o && p.R_o < p.R_n)) fail("opening_radius out of range");
  if (!(p.R_o <= p.R_b && p.R_b < p.R_n)) fail("bleb_radius out of range");
  Geometry g = make_geometry(p.R_n, p.R_o, p.R_b);

  // chromatin data (chrdat.cu:40-63)
  p.T = pm.get<float>("temperature", 298.0f);
  if (p.preset == PRESET_BASELINE) {
    p.lbs_area_fraction = pm.get<float>("lbs_area_fraction", 0.25f);
    float noacf = 2.0f / (1.0f + g.noc);
    const float depth = std::pow(2.0f, 1.0f / 6.0f);
    uint32_t nl_def = (uint32_t)std::floor(
        p.lbs_area_fraction * 4.0 / std::pow(CCP_LCO / (p.R_n - depth), 2.0) * noacf);
    p.n_l = pm.get<uint32_t>("number_of_lbs", nl_def);
  } else {
    p.n_l = pm.get<uint32_t>("number_of_lbs", 0u);
  }
  p.fpf = pm.get<uint32_t>("frames_per_file", 128u);
  const uint32_t n_max = p.relaxed ? (1u << 28) : 100000u;
  if (!(1 <= p.N && p.N < n_max)) fail("number_of_particles out of range");
  if (!(0.0f <= p.T && p.T < 1000.0f)) fail("temperature out of range");
  if (!(p.n_l < (p.relaxed ? (1u << 24) : 100000u))) fail("number_of_lbs out of range");
  if (!(1 <= p.fpf && p.fpf < 10000)) fail("frames_per_file out of range");
  float cvf = p.N * std::pow((CCP_RCO / 2.0) / (p.R_n - (CCP_RCO / 2.0)), 3.0);
  if (cvf > 0.4f) fail("chromatin volume fraction above 0.4");
  float noacf = 2.0f / (1.0f + g.noc);
  float laf = noacf * p.n_l * std::pow(CCP_LCO / (p.R_n - CCP_RCO), 2.0) / 4.0;
  if (laf > 0.4f) fail("lbs area fraction above 0.4");

  // force field
  if (p.preset == PRESET_CCP) {
    p.ff = preset_ccp(p.T);
  } else {
    float kT = pm.get<float>("kT", 1.0f);
    float dt = pm.get<float>("timestep", 1.0e-3f);
    if (!(kT >= 0.0f && kT < 100.0f)) fail("kT out of range");
    if (!(dt > 0.0f && dt < 0.1f)) fail("timestep out of range");
    p.ff = preset_baseline(kT, dt);
  }

  // simulation (chrsim.cu:421-435)
  p.spf = pm.get<uint32_t>("steps_per_frame", (uint32_t)(1.0 / p.ff.dt + 0.5));
  p.tpb = pm.get<uint32_t>("threads_per_block", 128u);
  if (!(1 <= p.spf && p.spf < 10000)) fail("steps_per_frame out of range");
  if (!(1 <= p.tpb && p.tpb < 1025)) fail("threads_per_block out of range");

  // engine keys
  p.seed = pm.get<uint64_t>("seed", 0ull);
  if (p.preset == PRESET_CCP) {
    p.n_chains = pm.get<int>("number_of_chains", p.N == CCP_N_DEF ? 12 : 1);
    p.contact_cutoff = pm.get<float>("contact_cutoff", CCP_ACO);
    p.contact_bins = pm.get<int>("contact_bins", 0);
  } else {
    p.n_chains = pm.get<int>("number_of_chains", 1);
    p.contact_cutoff = pm.get<float>("contact_cutoff", 1.5f);
    p.contact_bins = pm.get<int>("contact_bins", (int)std::min<uint32_t>(p.N, 2048u));
  }
  p.lad_fraction = pm.get<float>("lad_fraction", 0.1f);
  p.mean_block = pm.get<float>("mean_block_length", 16.0f);
  p.sequence_file = pm.get<std::string>("sequence_file", p.sequence_file);
  // the typed layout pays off when the repulsive cutoff is below the cell side
  // (baseline cells of 1.25 sigma); ccp's cells of aco = 2 sigma gain nothing
  p.pair_kernel = pm.get<int>("pair_kernel", p.preset == PRESET_BASELINE ? 4 : 2);
  if (!(p.pair_kernel >= 0 && p.pair_kernel <= 4)) fail("pair_kernel out of range");
  p.pair_lanes = pm.get<int>("pair_lanes", 0);  // 0: by the batch's bead count
  if (!(p.pair_lanes == 0 || p.pair_lanes == 1 || p.pair_lanes == 2 || p.pair_lanes == 4 ||
        p.pair_lanes == 8))
    fail("pair_lanes out of range");
  p.persistent = pm.get<int>("persistent", 0);
  if (!(p.persistent == 0 || p.persistent == 1)) fail("persistent out of range");
  if (!(p.n_chains >= 1 && (uint32_t)p.n_chains <= p.N)) fail("number_of_chains out of range");
  if (!(p.contact_cutoff > 0.0f)) fail("contact_cutoff out of range");
  if (p.contact_bins < 0) fail("contact_bins out of range");
  if (!(p.lad_fraction >= 0.0f && p.lad_fraction <= 1.0f)) fail("lad_fraction out of range");
  if (!(p.mean_block >= 1.0f)) fail("mean_block_length out of range");
  float need = std::max({p.ff.rc_att, p.ff.rc_rep, p.ff.rc_icg, p.contact_cutoff, p.ff.mis});
  // cells of half the largest cutoff with the 5x5x5 half-shell stencil: for
  // ccp (whose own grid has side aco = 2, chrsim.cu:425) 15-20 % faster per
  // step than cells of aco on one system of 8192-99000 beads (GB300)
  float def_cs = (p.pair_kernel >= 2) ? 0.5f * need : need;
  p.cell_side = pm.get<float>("cell_side", def_cs);
  // cells of at least the largest cutoff use the 3x3x3 neighbourhood; cells of
  // at least half of it the 5x5x5 one (half-shell pair kernel only)
  if (!(p.cell_side < 1.0e3f)) fail("cell_side below interaction cutoff");
  if (p.cell_side >= need)
    p.reach = 1;
  else if (p.cell_side >= 0.5f * need && p.pair_kernel >= 2)
    p.reach = 2;
  else
    fail("cell_side below interaction cutoff");
  return p;
}

// ------------------------------------------------------------ host RNG

HostRng::HostRng(uint64_t seed, uint32_t stream_id)
    : k0((uint32_t)seed), k1((uint32_t)(seed >> 32)) {
  ctr = (uint64_t)stream_id << 40;
}

uint32_t HostRng::next_u32() {
  if (left == 0) {
    U32x4 c{(uint32_t)ctr, (uint32_t)(ctr >> 32), STREAM_INIT << 16, 0x1C0DEu};
    U32x4 o = philox4x32_10(c, k0, k1);
    buf[0] = o.x;
    buf[1] = o.y;
    buf[2] = o.z;
    buf[3] = o.w;
    ++ctr;
    left = 4;
  }
  return buf[4 - left--];
}

float HostRng::uniform() { return u01_open0(next_u32()); }

// ------------------------------------------------------------ initial condition

namespace {
struct V3 {
  float x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float len(V3 a) { return std::sqrt(dot(a, a)); }

V3 random_direction(HostRng &rng) {
  float ran = rng.uniform();
  float theta = std::acos(1.0 - 2.0 * ran);
  ran = rng.uniform();
  float phi = 2.0 * M_PI * ran;
  return {(float)(std::sin(theta) * std::cos(phi)), (float)(std::sin(theta) * std::sin(phi)),
          (float)std::cos(theta)};
}
}  // namespace

// chrsim::set_lbs_positions (chrsim.cu:596-631): uniform directions at radius
// R_n - depth, rejected within 2 lco of an earlier site or in the opening cap.
void place_lbs(const Geometry &g, float lbs_depth, float lco, int n_l, HostRng &rng,
               std::vector<float> &xyz) {
  xyz.assign((size_t)3 * n_l, 0.0f);
  const float h = 2.0f * lco;  // hash cell = exclusion distance
  std::unordered_map<int64_t, std::vector<int>> grid;
  auto key = [&](int a, int b, int c) {
    return ((int64_t)(a + (1 << 20)) << 42) | ((int64_t)(b + (1 << 20)) << 21) | (c + (1 << 20));
  };
  long long rejects = 0;
  for (int i = 0; i < n_l;) {
    V3 d = random_direction(rng);
    V3 p = (g.R_n - lbs_depth) * d;
    bool ok = true;
    if (p.z / len(p) > g.noc) ok = false;
    int cx = (int)std::floor(p.x / h), cy = (int)std::floor(p.y / h), cz = (int)std::floor(p.z / h);
    for (int a = -1; a <= 1 && ok; ++a)
      for (int b = -1; b <= 1 && ok; ++b)
        for (int c = -1; c <= 1 && ok; ++c) {
          auto it = grid.find(key(cx + a, cy + b, cz + c));
          if (it == grid.end()) continue;
          for (int j : it->second) {
            V3 q{xyz[3 * j], xyz[3 * j + 1], xyz[3 * j + 2]};
            if (len(q - p) < 2.0f * lco) {
              ok = false;
              break;
            }
          }
        }
    if (!ok) {
      if (++rejects > 200000000LL) throw Error(ST_PARAM, "unable to place lamina binding sites");
      continue;
    }
    xyz[3 * i] = p.x;
    xyz[3 * i + 1] = p.y;
    xyz[3 * i + 2] = p.z;
    grid[key(cx, cy, cz)].push_back(i);
    ++i;
  }
}

// chrsim::set_particle_types (chrsim.cu:634-675).
void make_types_ccp(uint32_t N, const std::string &seq_file, HostRng &rng,
                    std::vector<int32_t> &pt) {
  pt.assign(N, 1);
  if (N == CCP_N_DEF) {
    std::ifstream f(seq_file);
    if (!f.is_open()) throw Error(ST_IO, "unable to open " + seq_file);
    char c;
    for (uint32_t i = 0; i < N; ++i) {
      f >> c;
      pt[i] = (c == 'A') ? 0 : 1;
    }
    if (f.fail()) throw Error(ST_IO, "failed to read sequence");
    return;
  }
  uint32_t cde = 0;
  int32_t cpt = 1;
  for (uint32_t i = 0; i < N; ++i) {
    if (i == cde) {
      float edl;
      do {
        float ran = rng.uniform();
        edl = -CCP_MDL * std::log(ran);
      } while ((edl / CCP_MDL) > 5 || edl < 1.0f);
      cde = (uint32_t)(i + edl);
      cpt = (cpt == 0) ? 1 : 0;
    }
    pt[i] = cpt;
  }
}

// Two-state Markov sequence with mean block length mean_block and an
// independent lamina-binding flag on a fraction lad_fraction of the beads.
void make_types_markov(int N, float mean_block, float lad_fraction, HostRng &rng,
                       std::vector<int32_t> &pt) {
  pt.assign(N, 1);
  int32_t cur = rng.uniform() <= 0.5f ? 0 : 1;
  const float p_switch = 1.0f / mean_block;
  for (int i = 0; i < N; ++i) {
    if (i > 0 && rng.uniform() <= p_switch) cur ^= 1;
    int32_t v = cur;
    if (rng.uniform() <= lad_fraction) v |= 2;
    pt[i] = v;
  }
}

// ------------------------------------------------------------ formats

// cnfs (util.cuh:91-104): width, fill and fixed precision.
static std::string cnfs_f(double v, int w, int prc) {
  std::stringstream s;
  s << std::setw(w) << std::setprecision(prc) << std::fixed << v;
  return s.str();
}

// chrdat::write_frame_txt (chrdat.cu:107-133).
std::string format_frame_txt(uint32_t i_f, float t, const std::vector<int32_t> &pt,
                             const float *xyz, int N) {
  std::ostringstream o;
  o << i_f << " " << t << "\n";
  o << std::setw(5) << N << "\n";
  for (int i = 0; i < N; ++i) {
    char c = ((pt[i] & 1) == 0) ? 'A' : 'B';
    o << std::setw(5) << i + 1 << std::left << std::setw(5) << c;
    o << std::right << std::setw(5) << c << std::setw(5) << i + 1;
    o << cnfs_f(xyz[3 * i], 8, 3) << cnfs_f(xyz[3 * i + 1], 8, 3) << cnfs_f(xyz[3 * i + 2], 8, 3);
    o << "\n";
  }
  o << cnfs_f(0.0, 10, 5) << cnfs_f(0.0, 10, 5) << cnfs_f(0.0, 10, 5) << "\n";
  return o.str();
}

// chrdat::write_lbs_txt (chrdat.cu:229-254).
std::string format_lbs_txt(const float *xyz, int n_l) {
  std::ostringstream o;
  o << "\n";
  o << std::setw(5) << n_l << "\n";
  for (int i = 0; i < n_l; ++i) {
    o << std::setw(5) << i + 1 << std::left << std::setw(5) << 'C';
    o << std::right << std::setw(5) << 'C' << std::setw(5) << i + 1;
    o << cnfs_f(xyz[3 * i], 8, 3) << cnfs_f(xyz[3 * i + 1], 8, 3) << cnfs_f(xyz[3 * i + 2], 8, 3);
    o << "\n";
  }
  o << cnfs_f(0.0, 10, 5) << cnfs_f(0.0, 10, 5) << cnfs_f(0.0, 10, 5) << "\n";
  return o.str();
}

// chrdat::write_frame_bin (chrdat.cu:168-201): minimal little-endian .trr frame.
std::string format_trr_frame(uint32_t i_f, float t, const float *xyz, int N) {
  uint32_t tb;
  std::memcpy(&tb, &t, 4);
  uint32_t h[18] = {1993, 1, 0, 0, 0, 0, 0, 0, 0, 0, 3u * (uint32_t)N * 4u, 0, 0,
                    (uint32_t)N, i_f, 0, tb, 0};
  std::string s(sizeof(h) + (size_t)12 * N, '\0');
  std::memcpy(&s[0], h, sizeof(h));
  std::memcpy(&s[sizeof(h)], xyz, (size_t)12 * N);
  return s;
}

// chrsim::save_checkpoint (chrsim.cu:525-536).
std::string format_checkpoint(uint32_t i_f, float t, const std::vector<int32_t> &pt,
                              const float *xyz, int N, const float *lxyz, int n_l) {
  std::string s(8 + (size_t)4 * N + (size_t)12 * N + (size_t)12 * n_l, '\0');
  char *d = &s[0];
  std::memcpy(d, &i_f, 4);
  std::memcpy(d + 4, &t, 4);
  std::memcpy(d + 8, pt.data(), (size_t)4 * N);
  std::memcpy(d + 8 + (size_t)4 * N, xyz, (size_t)12 * N);
  if (n_l) std::memcpy(d + 8 + (size_t)16 * N, lxyz, (size_t)12 * n_l);
  return s;
}

// chrsim::load_checkpoint (chrsim.cu:539-555).
bool parse_checkpoint(const void *buf, size_t len, int N, int n_l, uint32_t &i_f, float &t,
                      std::vector<int32_t> &pt, std::vector<float> &xyz,
                      std::vector<float> &lxyz) {
  size_t need = 8 + (size_t)16 * N + (size_t)12 * n_l;
  if (len < need) return false;
  const char *s = (const char *)buf;
  std::memcpy(&i_f, s, 4);
  std::memcpy(&t, s + 4, 4);
  pt.resize(N);
  xyz.resize((size_t)3 * N);
  lxyz.resize((size_t)3 * n_l);
  std::memcpy(pt.data(), s + 8, (size_t)4 * N);
  std::memcpy(xyz.data(), s + 8 + (size_t)4 * N, (size_t)12 * N);
  if (n_l) std::memcpy(lxyz.data(), s + 8 + (size_t)16 * N, (size_t)12 * n_l);
  return true;
}

// chrdat::read_frame_txt (chrdat.cu:136-165), token by token.
bool parse_frame_txt(const std::string &text, int N, uint32_t &i_f, float &t,
                     std::vector<int32_t> &pt, std::vector<float> &xyz) {
  std::istringstream is(text);
  std::string aux;
  char c;
  is >> i_f >> t;
  is >> aux;
  pt.resize(N);
  xyz.resize((size_t)3 * N);
  for (int i = 0; i < N; ++i) {
    is >> aux;
    is >> c >> aux;
    pt[i] = (c == 'A') ? 0 : 1;
    is >> xyz[3 * i] >> xyz[3 * i + 1] >> xyz[3 * i + 2];
  }
  is >> aux >> aux >> aux;
  return !is.fail();
}

// Reads the layout written by format_lbs_txt: count line, then per site the
// index+name token, the name token+index, x, y, z.
bool parse_lbs_txt(const std::string &text, int n_l, std::vector<float> &xyz) {
  std::istringstream is(text);
  std::string aux;
  char c;
  int n = -1;
  is >> n;
  if (is.fail() || n != n_l) return false;
  xyz.resize((size_t)3 * n_l);
  for (int i = 0; i < n_l; ++i) {
    is >> aux;
    is >> c >> aux;
    is >> xyz[3 * i] >> xyz[3 * i + 1] >> xyz[3 * i + 2];
  }
  is >> aux >> aux >> aux;
  return !is.fail();
}

}  // namespace ccpgpu
