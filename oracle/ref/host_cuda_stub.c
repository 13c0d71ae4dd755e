/* Host-only stand-ins for the CUDA runtime calls made by the reference's host
 * code (Program/src/chrdat.cu, chrana.cu, util.cu), so that its analysis loops
 * run here on the host cores without a GPU. TEST INFRASTRUCTURE: linked only
 * into oracle/_ref/chrana_driver by oracle/ref/build_chrana.sh.
 *
 * Device allocations are zeroed host allocations, copies are memmove, and
 * kernel launches and registrations do nothing: the driver reads only the
 * observables that chrana::calc_observables computes on the host
 * (chrana.cu:371-480), never the outputs of the kernels it launches. The
 * registration and launch hooks are declared without a parameter list; they
 * ignore their arguments and return success. */
#include <stdlib.h>
#include <string.h>

int cudaMalloc(void **p, size_t n) {
  *p = calloc(n ? n : 1, 1);
  return *p ? 0 : 2;
}

int cudaHostAlloc(void **p, size_t n, unsigned int flags) {
  (void)flags;
  return cudaMalloc(p, n);
}

int cudaFree(void *p) {
  free(p);
  return 0;
}

int cudaFreeHost(void *p) {
  free(p);
  return 0;
}

int cudaMemcpy(void *dst, const void *src, size_t n, int kind) {
  (void)kind;
  memmove(dst, src, n);
  return 0;
}

const char *cudaGetErrorString(int e) {
  (void)e;
  return "host stand-in of the CUDA runtime";
}

static void *fat_handle;

void **__cudaRegisterFatBinary() { return &fat_handle; }
void __cudaRegisterFatBinaryEnd() {}
void __cudaUnregisterFatBinary() {}
void __cudaRegisterFunction() {}
void __cudaRegisterVar() {}
unsigned __cudaPushCallConfiguration() { return 0; }
int __cudaPopCallConfiguration() { return 0; }
int __cudaGetKernel() { return 0; }
int __cudaLaunchKernel() { return 0; }
