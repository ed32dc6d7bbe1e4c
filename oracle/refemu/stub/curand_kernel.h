/* Stand-in for <curand_kernel.h> in the serial host emulation of the
 * reference kernels.  The reference only declares a curandState pointer and
 * calls curand_init from a kernel it never launches. */
#ifndef PF_STUB_CURAND_KERNEL_H
#define PF_STUB_CURAND_KERNEL_H
typedef struct {
  unsigned long long s;
} curandState;
static inline void curand_init(unsigned long long seed, unsigned long long seq,
                               unsigned long long off, curandState *st) {
  st->s = seed ^ (seq << 1) ^ off;
}
#endif
