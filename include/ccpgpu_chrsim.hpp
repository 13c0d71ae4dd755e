// Header-only drop-in for ccp's simulation class over the C ABI of libccpgpu.
//
// Replaces Program/src/chrsim.cuh: the class mmc::chrsim (chrsim.cuh:36-100,
// and the frame I/O it inherits from mmc::chrdat, chrdat.cuh:81-100) with the
// same public member functions, and the constants dt and mis
// (chrsim.cuh:18-20) that ccp's programs read, so ccp-perform.cu
// (Program/src/ccp-perform.cu:48-111) and ccp-profile.cu (:55-86) compile
// unchanged. It relies on the caller's own mmc::parmap, mmc::error and
// mmc::logger (Program/src/util.cuh:20-80) and, in ccp, on chrdat.cuh for the
// model constants (rco, lco): a maintainer replaces the body of chrsim.cuh with
//   #include "chrdat.cuh"
//   #include "ccpgpu_chrsim.hpp"
// Streams are filled from the byte images the library returns.
#ifndef CCPGPU_CHRSIM_HPP
#define CCPGPU_CHRSIM_HPP

#include <cstdint>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iterator>
#include <sstream>
#include <string>
#include <vector>

#include "ccpgpu.h"

namespace mmc {

// ccp's timestep and minimum initial separation (chrsim.cuh:18-20);
// ccp-profile.cu:82 turns frames into steps with dt. The engine's ccp preset
// uses the same values.
static constexpr float dt = 1.0 / 2048;
static constexpr float mis = 0.838732;

class chrsim {
 public:
  // chrsim::chrsim(parmap&) (chrsim.cu:421-455): the parameter map is handed
  // to the engine as the text of adjustable-parameters.dat. Like ccp
  // (chrsim.cu:454), the noise is seeded with the time unless the file has a
  // "seed" key.
  explicit chrsim(parmap &par) {
    std::string text;
    for (const auto &kv : par) text += kv.first + " " + kv.second + "\n";
    check(ccpgpu_create(text.c_str(), (uint64_t)std::time(nullptr), &h_));
  }
  ~chrsim() { ccpgpu_destroy(h_); }
  chrsim(const chrsim &) = delete;
  chrsim &operator=(const chrsim &) = delete;

  // chrsim::generate_initial_condition (chrsim.cu:470-522)
  void generate_initial_condition() {
    check(ccpgpu_generate_initial_condition(h_));
    logger::record("initial condition generated");
  }

  // chrsim::save_checkpoint / load_checkpoint (chrsim.cu:525-555)
  void save_checkpoint(std::ofstream &f) {
    write_bytes(f, &ccpgpu_checkpoint);
    logger::record("simulation checkpoint saved");
  }
  void load_checkpoint(std::ifstream &f) {
    std::vector<char> b((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    check(ccpgpu_load_checkpoint(h_, 0, b.data(), b.size()));
    logger::record("simulation checkpoint loaded");
  }

  // chrsim::run_simulation (chrsim.cu:558-593): one .trr frame per frame.
  void run_simulation(std::ofstream &f) {
    check(ccpgpu_run_simulation(h_, &frame_cb, &f));
    if (f.fail()) throw error("failed to write frame to binary file");
    logger::record("simulation ended");
  }

  // chrdat::write_frame_txt / write_lbs_txt / write_frame_bin (chrdat.cu:107-254)
  void write_frame_txt(std::ofstream &f) { write_bytes(f, &ccpgpu_frame_txt); }
  void write_lbs_txt(std::ofstream &f) { write_bytes(f, &ccpgpu_lbs_txt); }
  void write_frame_bin(std::ofstream &f) { write_bytes(f, &ccpgpu_frame_trr); }

  // chrdat::read_frame_txt (chrdat.cu:136-165)
  void read_frame_txt(std::ifstream &f) {
    std::string s((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    check(ccpgpu_read_frame_txt(h_, 0, s.data(), s.size()));
  }

  ccpgpu_sim *handle() { return h_; }

 private:
  ccpgpu_sim *h_ = nullptr;

  static void check(int rc) {
    if (rc != CCPGPU_OK) throw error(ccpgpu_last_error());
  }

  template <typename Fn>
  void write_bytes(std::ofstream &f, Fn fn) {
    size_t n = 0;
    fn(h_, 0, nullptr, 0, &n);
    std::vector<char> b(n);
    check(fn(h_, 0, b.data(), b.size(), &n));
    f.write(b.data(), (std::streamsize)n);
  }

  // .trr frame (chrdat.cu:174-194) of the positions handed over per frame
  static int frame_cb(void *user, uint32_t i_f, float t, const float *xyz, int32_t n) {
    std::ofstream &f = *static_cast<std::ofstream *>(user);
    uint32_t tb;
    static_assert(sizeof(tb) == sizeof(t), "float is 32-bit");
    std::memcpy(&tb, &t, 4);
    uint32_t h[18] = {1993, 1, 0, 0, 0, 0, 0, 0, 0, 0, 3u * (uint32_t)n * 4u, 0, 0,
                      (uint32_t)n, i_f, 0, tb, 0};
    f.write(reinterpret_cast<const char *>(h), sizeof(h));
    f.write(reinterpret_cast<const char *>(xyz), (std::streamsize)(12 * (size_t)n));
    return f.fail() ? 1 : 0;
  }
};

}  // namespace mmc

#endif  // CCPGPU_CHRSIM_HPP
