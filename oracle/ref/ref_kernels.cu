// Device image of the reference's own force, cell-list and analysis code —
// TEST INFRASTRUCTURE ONLY (it pins the oracle).
//
// This file contains no reference code: it #includes the reference's
// translation units where they lie (Program/src/chrsim.cu, sugrid.cu and
// chrana.cu, found through -I) and adds two extern "C" kernels whose bodies
// call the reference's own __device__ functions in the order of exec_RK_1
// (chrsim.cu:378-384) without the position update:
//   ref_forces_dst / ref_forces_icg: f[i] += calc_bf + calc_cf<T> + calc_srf<T>.
// The reference's own __global__ kernels calc_indexes, set_cells_empty,
// find_cells_limits (sugrid.cu:15-77), calc_cm and calc_sd_cp
// (chrana.cu:13-84) are compiled unchanged and looked up by their mangled
// names. Compiled with `nvcc -cubin` (device code only) by oracle/ref/build_ref.sh.
#include "chrana.cu"
#include "chrsim.cu"
#include "sugrid.cu"

extern "C" __global__ void ref_forces_dst(const unsigned int N, const mmc::cngeom ng,
                                          mmc::ptype *pt, mmc::vec3f *r, mmc::vec3f *f,
                                          mmc::vec3f *lr, mmc::sugrid *pgp,
                                          mmc::sugrid *lgp) {
  unsigned int i_p = blockIdx.x * blockDim.x + threadIdx.x;
  if (i_p >= N) return;
  mmc::calc_bf(N, pt, i_p, r, f);
  mmc::calc_cf<mmc::DST>(ng, i_p, r, f);
  mmc::calc_srf<mmc::DST>(pt, lr, pgp, lgp, i_p, r, f);
}

extern "C" __global__ void ref_forces_icg(const unsigned int N, const mmc::cngeom ng,
                                          mmc::ptype *pt, mmc::vec3f *r, mmc::vec3f *f,
                                          mmc::vec3f *lr, mmc::sugrid *pgp,
                                          mmc::sugrid *lgp) {
  unsigned int i_p = blockIdx.x * blockDim.x + threadIdx.x;
  if (i_p >= N) return;
  mmc::calc_bf(N, pt, i_p, r, f);
  mmc::calc_cf<mmc::ICG>(ng, i_p, r, f);
  mmc::calc_srf<mmc::ICG>(pt, lr, pgp, lgp, i_p, r, f);
}
