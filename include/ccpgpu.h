/*
 * ccpgpu — C ABI of the GB300 Brownian-dynamics engine for the ccp chromatin
 * model (Marco-Mendivil-Carboni/TFM, Program/src).
 *
 * The reference has no plugin or FFI layer: its simulation loop is the C++
 * class mmc::chrsim (Program/src/chrsim.cuh:36-56), which inherits the frame
 * I/O of mmc::chrdat (Program/src/chrdat.cuh:81-100) and is driven by main()
 * in Program/src/ccp-perform.cu:48-111 and Program/src/ccp-profile.cu:74-82.
 * Each entry point below names the member function it replaces. Streams
 * cannot cross a C ABI, so file I/O is offered both as byte buffers (for the
 * header-only mmc::chrsim shim in ccpgpu_chrsim.hpp, which writes them to the
 * caller's std::ofstream) and as the positions themselves.
 *
 * A handle owns all device memory, one CUDA stream and its CUDA graphs; no
 * device pointer crosses the ABI. Handles are independent; one handle must not
 * be used from two threads at once. Every function returns CCPGPU_OK (0) or an
 * error code; ccpgpu_last_error() returns the message of the last failure of
 * the calling thread (ccp's own message text for parameter range errors).
 *
 * A handle holds a batch of independent systems (replicas). A ccp run is a
 * batch of one system created from ccp's parameter file by ccpgpu_create.
 */
#ifndef CCPGPU_H
#define CCPGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CCPGPU_OK 0
#define CCPGPU_ERR_PARAM 1 /* parameter out of range (ccp's message)      */
#define CCPGPU_ERR_CUDA 2  /* CUDA runtime error ("cuda: <text>")         */
#define CCPGPU_ERR_IO 3    /* malformed file or buffer too small          */
#define CCPGPU_ERR_STATE 4 /* non-finite or escaped bead detected         */
#define CCPGPU_ERR_ARG 5   /* invalid argument (null pointer, bad index)  */

typedef struct ccpgpu_sim ccpgpu_sim;

typedef struct ccpgpu_info {
  int32_t n_systems;
  int32_t n_beads;      /* all systems */
  int32_t n_lbs;        /* all systems */
  int32_t n_chains;     /* all systems */
  int32_t n_cells;      /* all systems */
  int32_t preset;       /* 0 = ccp, 1 = baseline */
  uint32_t frames_per_file;
  uint32_t steps_per_frame;
  uint32_t frame_index; /* i_f of system 0 */
  float time;           /* t of system 0 */
  uint64_t step;        /* steps taken since step 0 */
  float dt, kT, noise_sd;
  float contact_cutoff;
  int32_t frames_observed;
  int32_t persistent_reach; /* 0: graph path; 1 or 2: steps run in the
                               persistent per-system kernel with that stencil */
} ccpgpu_info;

typedef struct ccpgpu_system_info {
  int32_t bead_offset, n_beads;
  int32_t chain_offset, n_chains;
  int32_t lbs_offset, n_lbs;
  int32_t cells_per_side;
  float cell_side;
  float nucleus_radius, opening_radius, bleb_radius;
  int32_t contact_bins;     /* side of the contact map */
  int32_t map_len;          /* beads of one copy that are binned */
  int32_t copy_len;         /* beads per chromosome copy */
  int32_t n_copies;         /* 2 for ccp's diploid N = 30386 model */
  int64_t map_offset;       /* offset of the packed map in the batch */
  uint64_t seed;
} ccpgpu_system_info;

/* Called once per trajectory frame by ccpgpu_run_simulation with the frame's
 * positions (3 floats per bead, chain order, system 0); a non-zero return
 * stops the run with CCPGPU_ERR_IO. */
typedef int (*ccpgpu_frame_fn)(void *user, uint32_t frame_index, float time,
                               const float *xyz, int32_t n_beads);

/* ---------------------------------------------------------------- lifetime */

/* chrsim::chrsim(parmap&) (chrsim.cu:421-455, chrdat.cu:13-88): parses ccp's
 * adjustable-parameters text, checks the ranges with ccp's messages and
 * allocates the system. seed keys the Philox noise (the reference seeds with
 * time(nullptr)); a "seed" key in the text takes precedence. */
int ccpgpu_create(const char *param_text, uint64_t seed, ccpgpu_sim **out);

/* Batch of n_systems independent systems sharing the force field and keys of
 * param_text. n_beads[i] >= 1 beads in n_chains[i] equal chains (NULL: the
 * number_of_chains key, else 1 chain; ccp's 30386-bead model defaults to, and
 * with 12 chains uses, its 12 chromosomes of chrdat.cuh:28-31, as ccpgpu_create does),
 * nucleus radius radii[i] (NULL: from the packing fraction or the
 * nucleus_radius key) and Philox seed seeds[i] (NULL: seed + i). No reference
 * counterpart: ccp runs replicas as separate processes (Scripts/makeallsim.py:105-121). */
int ccpgpu_batch_create(const char *param_text, int32_t n_systems, const int32_t *n_beads,
                        const int32_t *n_chains, const float *radii, const uint64_t *seeds,
                        uint64_t seed, ccpgpu_sim **out);

/* chrsim::~chrsim (chrsim.cu:458-467). */
int ccpgpu_destroy(ccpgpu_sim *h);

/* Message of the last failed call on this thread (mmc::error::what). */
const char *ccpgpu_last_error(void);

int ccpgpu_info_get(const ccpgpu_sim *h, ccpgpu_info *out);
int ccpgpu_system_info_get(const ccpgpu_sim *h, int32_t sys, ccpgpu_system_info *out);

/* ---------------------------------------------------------------- simulation */

/* chrsim::generate_initial_condition (chrsim.cu:470-522): LBS placement and
 * type sequence on the host, then the confined random walk and the
 * soft-repulsion relaxation on the GPU until no non-bonded pair is closer
 * than 0.838732. */
int ccpgpu_generate_initial_condition(ccpgpu_sim *h);

/* chrsim::set_particle_positons + perform_random_walk (chrsim.cu:678-802):
 * the confined random walk of every chain with the current types, without the
 * relaxation. ccp's 30386-bead diploid model walks its 12 chromosomes in cones
 * around shuffled icosahedral directions; other chains walk without a cone.
 * Chain c of a system draws attempt k from Philox4x32-10 keyed by the
 * system's seed with counter (k, c, 0x10057, 0x1C0DE). draws (NULL allowed,
 * n >= total chains) receives each chain's number of attempts. Returns
 * CCPGPU_ERR_STATE when a chain exceeds 256 attempts per bead + 2^17. */
int ccpgpu_random_walk(ccpgpu_sim *h, uint32_t *draws, size_t n);

/* chrsim::run_simulation (chrsim.cu:558-593): frames_per_file frames of
 * steps_per_frame Heun steps; after each frame i_f += 1, t += spf * dt and fn
 * receives the positions (fn may be NULL). Frame copies overlap the next
 * frame's steps. */
int ccpgpu_run_simulation(ccpgpu_sim *h, ccpgpu_frame_fn fn, void *user);

/* n_steps Heun steps of every system. When observe_every > 0 the observables
 * of ccpgpu_observe are accumulated every observe_every steps (at steps
 * step0, step0 + observe_every, ...). */
int ccpgpu_run_steps(ccpgpu_sim *h, uint64_t n_steps, uint32_t observe_every);

/* Enqueues n_steps Heun steps on the handle's stream and returns without
 * waiting or copying positions back (the device-resident form of
 * ccpgpu_run_steps); ccpgpu_synchronize waits and checks the error flags.
 * No reference counterpart (ccp's loop synchronises every frame, chrsim.cu:583). */
int ccpgpu_advance(ccpgpu_sim *h, uint64_t n_steps, uint32_t observe_every);
int ccpgpu_synchronize(ccpgpu_sim *h);

/* The handle's cudaStream_t, for callers that time or order work against it. */
int ccpgpu_stream_handle(ccpgpu_sim *h, void **stream);

/* Average device time in ms of each kernel of one Heun step (plus one
 * observation), measured with CUDA events around individual launches on the
 * handle's stream over reps steps: out[0] scan (3 launches), [1] scatter,
 * [2] pair, [3] update stage 1, [4] update stage 2, [5] contacts,
 * [6] observe. Leaves the simulation state advanced by reps steps. */
int ccpgpu_kernel_times(ccpgpu_sim *h, int32_t reps, double *out, size_t n);

/* Autotuner (no reference counterpart): for each half-shell pair kernel (2:
 * one cell grid; 4: A beads and the others in separate grids) and per size
 * class of the batch (bead counts in [2^k, 2^(k+1))) it times cell sides of 1,
 * 0.75, 0.625, 0.55 and 0.5 times the largest cutoff (the last four with the
 * 5x5x5 stencil), keeps the fastest per class, keeps the faster kernel, then
 * picks the per-bead tile size (64, 128, 256) and the lanes per bead (1, 2,
 * 4, 8; tile x lanes <= 512). Requires pair_kernel 2 or 4. Each
 * candidate runs reps steps; positions, time and the noise counter are
 * restored afterwards. report receives a NUL-terminated JSON summary (size in
 * *len; CCPGPU_ERR_IO when cap is too small, after tuning). */
int ccpgpu_autotune(ccpgpu_sim *h, int32_t reps, char *report, size_t cap, size_t *len);

/* Number of engine kernels launched since creation (graph nodes included). */
int ccpgpu_kernel_count(const ccpgpu_sim *h, uint64_t *count);

/* Device error flags: [0] non-finite position, [1] bead outside its grid,
 * [2] counting-sort slot outside its system, [3] noise truncation exhausted,
 * [4] random-walk draw budget exhausted.
 * clear != 0 resets them. Returns CCPGPU_ERR_STATE when [0] or [2] is set. */
int ccpgpu_error_flags(ccpgpu_sim *h, int32_t *flags8, int32_t clear);

/* ---------------------------------------------------------------- state */

/* Positions (3 floats per bead, chain order, all systems): chrdat's hr array
 * (chrdat.cuh:120) after cudaMemcpy D2H (chrsim.cu:583), and its upload. */
int ccpgpu_get_positions(ccpgpu_sim *h, float *xyz, size_t n_floats);
int ccpgpu_set_positions(ccpgpu_sim *h, const float *xyz, size_t n_floats);
/* Bead type codes of ccp's ptype enum (0 = A / LADh, 1 = B / LNDe); bit 1 is
 * the lamina-binding flag of the baseline preset. */
int ccpgpu_get_types(const ccpgpu_sim *h, int32_t *pt, size_t n);
int ccpgpu_set_types(ccpgpu_sim *h, const int32_t *pt, size_t n);
/* Lamina-binding sites (3 floats per site, all systems): chrdat's hlr. */
int ccpgpu_get_lbs(const ccpgpu_sim *h, float *xyz, size_t n_floats);
int ccpgpu_set_lbs(ccpgpu_sim *h, const float *xyz, size_t n_floats);
/* Total force on every bead at the current positions (production mode):
 * the f array of exec_RK_1 (chrsim.cu:381-384) before the position update. */
int ccpgpu_compute_forces(ccpgpu_sim *h, float *fxyz, size_t n_floats);

/* ---------------------------------------------------------------- formats */

/* Byte images of ccp's files for system sys. When buf is NULL or cap is too
 * small, *len receives the size and CCPGPU_ERR_IO is returned (len only).
 *   frame_txt   chrdat::write_frame_txt  (.gro, chrdat.cu:107-133)
 *   lbs_txt     chrdat::write_lbs_txt    (chrdat.cu:229-254)
 *   frame_trr   chrdat::write_frame_bin  (.trr frame, chrdat.cu:168-201)
 *   checkpoint  chrsim::save_checkpoint  (chrsim.cu:525-536) */
int ccpgpu_frame_txt(ccpgpu_sim *h, int32_t sys, char *buf, size_t cap, size_t *len);
int ccpgpu_lbs_txt(ccpgpu_sim *h, int32_t sys, char *buf, size_t cap, size_t *len);
int ccpgpu_frame_trr(ccpgpu_sim *h, int32_t sys, char *buf, size_t cap, size_t *len);
int ccpgpu_checkpoint(ccpgpu_sim *h, int32_t sys, void *buf, size_t cap, size_t *len);
/* chrsim::load_checkpoint (chrsim.cu:539-555) and chrdat::read_frame_txt
 * (chrdat.cu:136-165), chrdat::read_lbs_txt (chrdat.cu:257-284). */
int ccpgpu_load_checkpoint(ccpgpu_sim *h, int32_t sys, const void *buf, size_t len);
int ccpgpu_read_frame_txt(ccpgpu_sim *h, int32_t sys, const char *text, size_t len);
int ccpgpu_read_lbs_txt(ccpgpu_sim *h, int32_t sys, const char *text, size_t len);

/* ---------------------------------------------------------------- observables */

/* Accumulates one frame of observables at the current positions: contact map
 * counts (calc_cm, chrana.cu:48-84), contact counts by separation (the cp of
 * calc_sd_cp, chrana.cu:13-45), FP64 sums for Rg^2 and the radial bead
 * density (chrana.cu:372-480); with_sdist != 0 adds the FP64 spatial-distance
 * sums by separation (the sd of calc_sd_cp). */
int ccpgpu_observe(ccpgpu_sim *h, int32_t with_sdist);
int ccpgpu_reset_observables(ccpgpu_sim *h);
/* Packed lower-triangular contact counts of system sys, element
 * bx * (bx + 1) / 2 + by for bins bx >= by: ordered bead pairs within the
 * contact cutoff summed over observed frames, self pairs excluded (ccp's
 * per-frame pixel value is 1000 * (count + self) / (n_copies * px^2)). */
int ccpgpu_contact_counts(ccpgpu_sim *h, int32_t sys, int32_t *tri, size_t n);
/* Per-system FP64 sums: out[0..2] = sum of positions, out[3] = sum of |r|^2,
 * out[4 + t*64 + b] = bead volume in radial shell b for t = A, B, all. */
int ccpgpu_observable_sums(ccpgpu_sim *h, int32_t sys, double *out, size_t n);
/* Contact counts and FP64 distance sums by separation s = 0..L/2 of one chain. */
int ccpgpu_separation_counts(ccpgpu_sim *h, int32_t chain, int32_t *counts, double *dist,
                             size_t n);
/* Number of non-bonded pairs (|i - j| >= 2) closer than 0.838732 per system
 * (chrsim::particle_overlaps, chrsim.cu:805-820). */
int ccpgpu_overlaps(ccpgpu_sim *h, uint64_t *per_system, size_t n);

/* ---------------------------------------------------------------- analysis */

/* ccp-analyze's outputs (Program/src/ccp-analyze.cu:52-126), fed by the GPU
 * observables instead of re-read trajectory files. A simulation is what one
 * system runs between two ccpgpu_analysis_end_simulation calls (ccp-analyze:
 * one initial condition and its trajectories); in a batch each system is a
 * simulation. The frames share the observable buffers of ccpgpu_observe, so
 * do not observe otherwise (ccpgpu_observe, observe_every) during one. */

/* One frame of every system at the current positions (chrana::
 * calc_observables, chrana.cu:371-512): centre-of-mass distance, gyration
 * radius squared, nematic order parameter, nucleus chromatin fraction and
 * radial chromatin density join each system's time series; contact map,
 * contact probability and spatial distance by separation accumulate. */
int ccpgpu_analysis_frame(ccpgpu_sim *h);
/* The time series of system sys's current simulation: frames = its frame
 * count; with out, series k (0 dcm, 1 rg2, 2 nop, 3 ncf, 4 + t*64 + b the
 * radial density of type t = A, B, all in shell b) in out[k * frames ...].
 * n: capacity of out in floats. */
int ccpgpu_analysis_series(ccpgpu_sim *h, int32_t sys, float *out, size_t n, int32_t *frames);
/* Ends every system's simulation (calc_last_is_stat, clear_is_var,
 * chrana.cu:177-305): statistics of the series (sostat.cu:136-174:
 * thermalisation by the marginal standard error rule, standard error by
 * blocking), frame averages of the rest, and adds them to the combined
 * statistics. Clears the observable buffers. */
int ccpgpu_analysis_end_simulation(ccpgpu_sim *h);
/* analysis-XXX.dat of system sys's last simulation (save_last_is_stat,
 * chrana.cu:205-256): the byte image ccp-analyze writes. */
int ccpgpu_analysis_txt(ccpgpu_sim *h, int32_t sys, char *buf, size_t cap, size_t *len);
/* analysis-fin.dat over every simulation so far (calc_cs_final_stat +
 * save_cs_final_stat, chrana.cu:281-360, sostat.cu:176-224). The systems must
 * share size, chains, contact bins and radius. */
int ccpgpu_analysis_fin_txt(ccpgpu_sim *h, char *buf, size_t cap, size_t *len);
/* contact-map.bin: the packed lower-triangular contact-map averages over
 * every simulation so far as float64 (save_cm_avg_bin, chrana.cu:362-369). */
int ccpgpu_contact_map_bin(ccpgpu_sim *h, char *buf, size_t cap, size_t *len);

/* ---------------------------------------------------------------- no allocation */

/* Total force of one system evaluated without allocating device memory. No
 * counterpart in the reference. It is for callers that cannot call cudaMalloc
 * when they need forces: hosts whose own memory manager owns all of the GPU's
 * memory, or time-critical loops where the device synchronisation of
 * cudaMalloc/cudaFree would stall their other streams. The caller passes
 * device buffers: d_xyz (3 floats per bead), d_types (ccp type codes) and
 * d_forces (3 floats per bead, written), and the stream to run on (NULL: the
 * legacy default stream). The result equals ccpgpu_compute_forces for the same
 * system without lamina-binding sites (chain heads every n_beads / n_chains
 * beads, the preset's default force field and cell grid).
 *
 * Scratch: a static device array of about 2.9 MB inside the library, held by
 * every GPU that loads it until the process exits. Limits: n_beads <=
 * CCPGPU_NOALLOC_MAX_BEADS and cells_per_side^3 <= CCPGPU_NOALLOC_MAX_CELLS;
 * larger systems are rejected with CCPGPU_ERR_ARG. The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) and should come
 * before any stream capture on that device; the address is kept for the
 * process, so it is not valid after cudaDeviceReset on that device. The call
 * reports argument errors only: read the device flags of a call with
 * ccpgpu_noalloc_error_flags. Every call uses the same array and
 * it keeps the last call's contents: calls that overlap on the GPU (on
 * different streams without ordering) race and corrupt each other. */
#define CCPGPU_NOALLOC_MAX_BEADS 32768
#define CCPGPU_NOALLOC_MAX_CELLS 131072

typedef struct ccpgpu_noalloc_system {
  int32_t preset;       /* 0 = ccp, 1 = baseline */
  int32_t n_beads;      /* 3 .. CCPGPU_NOALLOC_MAX_BEADS */
  int32_t n_chains;     /* heads at c * (n_beads / n_chains); the last chain takes the rest */
  float nucleus_radius; /* spherical nucleus, finite and > 1 */
} ccpgpu_noalloc_system;

int ccpgpu_forces_noalloc(const ccpgpu_noalloc_system *sys, const float *d_xyz,
                          const int32_t *d_types, float *d_forces, void *stream);

/* The eight device flags (the layout of ccpgpu_error_flags) of the last
 * ccpgpu_forces_noalloc call on the current device; allocates nothing. Pass
 * the stream of that call: the copy is ordered after it and the function
 * waits for it. Returns CCPGPU_ERR_STATE when a position was not finite or a
 * cell slot inconsistent; flags8[1] reports a bead outside the nucleus's cell
 * grid (clamped to the border cell). Like the forces call, it shares the
 * static array, so a call overlapping another on the GPU reads its flags.
 * No counterpart in the reference (ccp throws from cuda_check, util.cu:83-91). */
int ccpgpu_noalloc_error_flags(int32_t *flags8, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* CCPGPU_H */
