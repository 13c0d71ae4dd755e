// Host-side pieces of the engine: the ccp parameter file, the two force-field
// presets, system construction, the initial-condition generator and ccp's
// file formats. Plain C++ (no CUDA types).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "common.cuh"

namespace ccpgpu {

// Error carrying one of the C-ABI status codes and ccp's message text.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

enum : int {
  ST_OK = 0,
  ST_PARAM = 1,
  ST_CUDA = 2,
  ST_IO = 3,
  ST_STATE = 4,
  ST_ARG = 5,
};

// ccp constants (chrdat.cuh:15-24, chrsim.cuh:18-20, chrana.cuh:16-18).
constexpr float CCP_K_B = 0.003356f;
constexpr float CCP_RCO = 1.154701f;
constexpr float CCP_ACO = 2.0f;
constexpr float CCP_MDL = 21.10139f;
constexpr float CCP_LCO = 0.5f;
constexpr float CCP_MIS = 0.838732f;
constexpr double CCP_DT = 1.0 / 2048;
constexpr uint32_t CCP_N_DEF = 30386;
constexpr int CCP_PX_SZ = 4;
constexpr uint32_t CCP_CHR_LIM[13] = {0,     2284,  4599,  6687,  9338,  12508, 15193,
                                      17477, 19792, 21880, 24531, 27701, 30386};

enum : int { PRESET_CCP = 0, PRESET_BASELINE = 1 };

// The ccp key/value parameter map: whitespace-separated pairs, the first
// occurrence of a key wins (util.cu:72-80 parmap, util.cuh:70-79 get_val).
struct ParamMap {
  std::vector<std::pair<std::string, std::string>> kv;
  explicit ParamMap(const std::string &text);
  bool has(const std::string &k) const;
  std::string raw(const std::string &k) const;
  template <typename T>
  T get(const std::string &k, T def) const;
};

// Resolved parameters of a run (ccp keys plus the engine's optional keys).
struct Params {
  int preset = PRESET_CCP;
  uint32_t N = CCP_N_DEF;
  float R_n = 0, R_o = 0, R_b = 0;
  float T = 298.0f;
  uint32_t n_l = 0;
  uint32_t fpf = 128, spf = 2048, tpb = 128;
  uint64_t seed = 0;
  int n_chains = 1;
  float contact_cutoff = CCP_ACO;
  int contact_bins = 0;  // 0: ccp pixels of 4 beads
  float cell_side = 0;   // 0: automatic
  int reach = 1;         // neighbour cells per axis: cell_side >= cutoff / reach
  float lad_fraction = 0.1f;
  float mean_block = 16.0f;
  float packing_fraction = 0.2f;
  float lbs_area_fraction = 0.25f;
  bool relaxed = false;
  // 0: full shell, thread per bead; 1: warp per cell (lane groups);
  // 2: half shell (Newton's third law), thread per bead
  int pair_kernel = 2;
  int pair_lanes = 0;  // lanes per bead of the half-shell pair kernels (0: by bead count)
  // 1: when every system fits one CTA's shared memory, steps run in the
  // persistent per-system kernel (one launch per frame); 0: graph path
  int persistent = 0;
  std::string sequence_file = "Program/data/sequence.txt";
  ForceField ff{};
};

// Parses and range-checks a ccp parameter text (chrdat.cu:13-63,
// chrsim.cu:421-435). Throws Error(ST_PARAM, ccp's message).
Params parse_params(const std::string &text);

// The calling thread's message for ccpgpu_last_error() (shared by every
// entry point of the library).
void set_last_error(const std::string &m);

// Force field of a preset with its default temperature and time step (ccp:
// T = 298 K, dt = 1/2048; baseline: kT = 1, dt = 1e-3); allocates nothing.
ForceField make_preset(int preset);

// One independent system of a batch.
struct SystemSpec {
  int n = 0;
  int n_chains = 1;
  std::vector<int> chain_first;  // optional explicit chain heads
  float R_n = 0, R_o = 0, R_b = 0;
  int n_lbs = 0;
  uint64_t seed = 0;
  int contact_bins = 0;
};

// Geometry derived from the radii (chrdat.cu:13-18).
struct Geometry {
  float R_n, R_o, R_b, noc, boc, nod, bod, d_b, d_m;
};
Geometry make_geometry(float R_n, float R_o, float R_b);

// Host Philox stream of (0, 1] uniforms for initial conditions.
struct HostRng {
  uint32_t k0, k1;
  uint64_t ctr = 0;
  uint32_t buf[4];
  int left = 0;
  explicit HostRng(uint64_t seed, uint32_t stream_id);
  uint32_t next_u32();
  float uniform();  // (0, 1]
};

// Host initial-condition pieces of one system (chrsim.cu:596-675); the
// confined random walk (chrsim.cu:678-802) runs on the GPU.
void place_lbs(const Geometry &g, float lbs_depth, float lco, int n_l, HostRng &rng,
               std::vector<float> &xyz);
void make_types_ccp(uint32_t N, const std::string &seq_file, HostRng &rng,
                    std::vector<int32_t> &pt);
void make_types_markov(int N, float mean_block, float lad_fraction, HostRng &rng,
                       std::vector<int32_t> &pt);

// ccp file formats (chrdat.cu:107-284, chrsim.cu:525-555, chrana.cu:363-369).
std::string format_frame_txt(uint32_t i_f, float t, const std::vector<int32_t> &pt,
                             const float *xyz, int N);
std::string format_lbs_txt(const float *xyz, int n_l);
std::string format_trr_frame(uint32_t i_f, float t, const float *xyz, int N);
std::string format_checkpoint(uint32_t i_f, float t, const std::vector<int32_t> &pt,
                              const float *xyz, int N, const float *lxyz, int n_l);
// Parses a checkpoint; returns false when the byte count does not match.
bool parse_checkpoint(const void *buf, size_t len, int N, int n_l, uint32_t &i_f, float &t,
                      std::vector<int32_t> &pt, std::vector<float> &xyz,
                      std::vector<float> &lxyz);
bool parse_frame_txt(const std::string &text, int N, uint32_t &i_f, float &t,
                     std::vector<int32_t> &pt, std::vector<float> &xyz);
bool parse_lbs_txt(const std::string &text, int n_l, std::vector<float> &xyz);

// ccp's bead type code (ptype enum, chrdat.cuh:40-44): 0 = A (LADh), 1 = B (LNDe).
// Bit 1 carries an explicit lamina-binding flag for the baseline preset.
inline uint32_t type_to_flags(int32_t pt, int preset) {
  uint32_t f = 0;
  bool a = (pt & 1) == 0;
  if (a) f |= BF_HET;
  if (preset == PRESET_CCP ? a : ((pt & 2) != 0)) f |= BF_LAD;
  return f;
}

}  // namespace ccpgpu
