// pf_common.cuh -- shared device definitions of the coupled step.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "pfgpu.h"

namespace pf {

// D3Q19 in the reference's ordering (LB_kernel.cu:40-47): the ordering is
// the fIN[19] layout at the boundary.
constexpr int Q = 19;
__host__ __device__ constexpr int cx(int d) {
  constexpr int v[Q] = {0, 1, -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0};
  return v[d];
}
__host__ __device__ constexpr int cy(int d) {
  constexpr int v[Q] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1};
  return v[d];
}
__host__ __device__ constexpr int cz(int d) {
  constexpr int v[Q] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1};
  return v[d];
}
__host__ __device__ constexpr double wgt(int d) {
  return d == 0 ? 1.0 / 3.0 : (d < 7 ? 1.0 / 18.0 : 1.0 / 36.0);
}
__host__ __device__ constexpr int opp(int d) {
  constexpr int v[Q] = {0, 2, 1, 4, 3, 6, 5, 12, 11, 14, 13, 8, 7, 10, 9, 18, 17, 16, 15};
  return v[d];
}

constexpr double kPi = 3.141592653589793;  // GPUDefines.h:36
constexpr int kBrickX = 32;                // force brick = 32 x-nodes of one row (one warp)
constexpr int kLbmBlock = 128;             // threads of an LBM CTA (4 bricks)
constexpr int kBinCap = 512;               // Morse cell-bin capacity
constexpr double kFixScale = 1099511627776.0;  // 2^40: fixed-point force accumulation

// Device error bits (set instead of trapping; the host reads them after a step)
enum : uint32_t {
  ERR_BIN_OVERFLOW = 1u,
  ERR_BOND_OVERFLOW = 2u,
  ERR_NONFINITE = 4u,
  ERR_MEMBRANE_SIZE = 8u,
  ERR_WAIT_TIMEOUT = 16u,  // a bounded wait on an mbarrier gave up
  ERR_FAR_FLAGGED = 32u,   // a force brick lay in the far region (a marker moved over a node)
  ERR_INPUT = 64u,         // caller-given device arrays inconsistent (membrane pass without allocation)
};

// Per-job device-resident control block: written by kernels, read by the host
// between steps.  Graph replays read the step counter from here.
struct Control {
  long long step;         // coupled steps completed
  int done;               // 1: platelet detached (semLB.cu:451-455); 2: stop step reached
  int first;              // next LBM step is the first after an upload
  int total_bond;         // sum of bond counts of the last bond pass
  unsigned int err;       // ERR_* bits
  int active_count[2];    // active-brick list lengths per force buffer
  int nops;               // bond slot operations of the last bond pass
  int pad;
  int nops_active[2];     // bond pass counters: operations, active receptors
  int occupied;           // Morse cells holding at least one element
  // pipelined far-region lattice pass: the step it computes next, and
  // whether that step is the first after an upload
  int far_first;
  long long far_step;
  // the step after which the job stops by itself (done = 2; 0: never)
  long long stop;
  // quiet lattice pass (bricks without force in the previous step): the
  // step it computes, whether that step is the first after an upload, and
  // whether to skip it (the job was done when the pass was scheduled).  Set
  // by the flagged-brick pass of the step before (the pass then runs ahead,
  // beside that step's moments and interpolation) or by the prologue.
  long long qstep;
  int qfirst;
  int qskip;
};

// ------------------------------------------------------------- Philox
// Philox-4x32-10 (Salmon et al., SC'11): published multipliers and Weyl
// constants, ten rounds.
__host__ __device__ inline void philox4x32(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}
__host__ __device__ inline double u53(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}
// Two uniforms of receptor `rid` at coupled step `step`.
__host__ __device__ inline void receptor_uniforms(uint64_t seed, long long step, long long rid, double& u1,
                                                  double& u2) {
  uint32_t c[4] = {(uint32_t)step, (uint32_t)((uint64_t)step >> 32), (uint32_t)rid,
                   (uint32_t)((uint64_t)rid >> 32) ^ 0x52454350u};
  philox4x32(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  u1 = u53(c[0], c[1]);
  u2 = u53(c[2], c[3]);
}
__host__ __device__ inline double detach_uniform(uint64_t seed, long long step) {
  uint32_t c[4] = {(uint32_t)step, (uint32_t)((uint64_t)step >> 32), 0xFFFFFFFFu, 0x44455443u};
  philox4x32(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  return u53(c[0], c[1]);
}

// ------------------------------------------------------------- storage
// Populations are stored shifted, g = f - w (FP16: q = g / (w * scale)).
template <class S>
struct StoreTraits;
template <>
struct StoreTraits<double> {
  __device__ static double load(const double* p, int, double) { return __ldg(p); }
  __device__ static void store(double* p, double v, int, double) { *p = v; }
};
template <>
struct StoreTraits<float> {
  __device__ static float load(const float* p, int, float) { return __ldg(p); }
  __device__ static void store(float* p, float v, int, float) { *p = v; }
};
template <>
struct StoreTraits<__half> {
  __device__ static float load(const __half* p, int, float s) { return __half2float(__ldg(p)) * s; }
  __device__ static void store(__half* p, float v, int, float inv_s) { *p = __float2half_rn(v * inv_s); }
};

// The job owning CTA b of a fused batch launch: the last j with
// start[j] <= b (jobs with no CTAs have start[j] == start[j + 1]).
__device__ __forceinline__ int batch_job_of(const int* start, int nj, int b) {
  int lo = 0, hi = nj;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (start[mid] <= b) lo = mid;
    else hi = mid;
  }
  return lo;
}

// word-parallel copy of a trivially copyable struct by the threads of a CTA
// (a fused batch kernel's per-job constants into shared memory)
template <class T>
__device__ __forceinline__ void cta_copy(T& dst, const T& src) {
  static_assert(sizeof(T) % 4 == 0, "word copy");
  for (int i = threadIdx.x; i < (int)(sizeof(T) / 4); i += blockDim.x)
    reinterpret_cast<int*>(&dst)[i] = reinterpret_cast<const int*>(&src)[i];
}

__device__ inline int wrapi(int a, int n) {
  int r = a % n;
  return r < 0 ? r + n : r;
}

}  // namespace pf
