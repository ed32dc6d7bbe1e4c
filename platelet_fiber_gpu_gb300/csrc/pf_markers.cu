// pf_markers.cu -- kernels on immersed markers (platelet elements and fibrin
// nodes): IBM spreading and interpolation (LB_kernel.cu:1419-1642, restated
// element-centric over the 4x4x4 stencil), position update
// (sem_kernel.cu:2087-2148), the per-platelet membrane force pass
// (sem_kernel.cu:320-1749), Morse pair forces over cell bins, fibrin link
// forces (fiber.cpp:647-733) and the receptor-bond pass
// (sem_kernel.cu:1750-2083).
#include <algorithm>

#include "pf_internal.h"

namespace pf {

namespace {

__device__ __forceinline__ void atomic_add3(float4* F, size_t n, float x, float y, float z) {
  atomicAdd(F + n, make_float4(x, y, z, 0.f));
}
__device__ __forceinline__ void atomic_add3(D4* F, size_t n, double x, double y, double z) {
  double* p = reinterpret_cast<double*>(F + n);
  atomicAdd(p, x);
  atomicAdd(p + 1, y);
  atomicAdd(p + 2, z);
}

// Nodes of one axis within 2 dx of x, with weights.
// FP64 build: the reference's arithmetic -- spreading forms node coordinates
// as int*float (LB_kernel.cu:1474), interpolation as int*double (:1581), and
// the support test is |x - x_i| < 2 dx in microns.
// FP32 build: one FP64 multiply to lattice units, then FP32 offsets (both
// IBM directions share one stencil).
template <class R>
struct Stencil;
template <>
struct Stencil<double> {
  static __device__ __forceinline__ int axis(double x, float dxf, double, int n, int wrap, int spread, int node[5],
                                             double w[5]) {
    const double dxd = (double)dxf;
    const double thr = spread ? (double)(2.0f * dxf) : 2.0 * dxd;
    const int base = (int)floor(x / dxd);
    int cnt = 0;
#pragma unroll
    for (int ii = base - 2; ii <= base + 2; ++ii) {
      const double xn = spread ? (double)((float)ii * dxf) : (double)ii * dxd;
      const double dd = x - xn;
      if (fabs(dd) >= thr) continue;
      int nd = ii;
      if (ii < 0 || ii >= n) {
        if (!wrap) continue;
        nd = wrapi(ii, n);
      }
      node[cnt] = nd;
      w[cnt] = 0.25 * (1.0 + cos(0.5 * kPi * dd / dxd));
      cnt++;
    }
    return cnt;
  }
};
template <>
struct Stencil<float> {
  static __device__ __forceinline__ int axis(double x, float, double inv_dx, int n, int wrap, int, int node[5],
                                             float w[5]) {
    const double r = x * inv_dx;
    const double fb = floor(r);
    const int base = (int)fb;
    const float fr = (float)(r - fb);
    int cnt = 0;
#pragma unroll
    for (int o = -1; o <= 2; ++o) {
      const float dd = fr - (float)o;
      if (!(fabsf(dd) < 2.f)) continue;
      int nd = base + o;
      if (nd < 0 || nd >= n) {
        if (!wrap) continue;
        nd = wrapi(nd, n);
      }
      node[cnt] = nd;
      w[cnt] = 0.25f * (1.f + cospif(0.5f * dd));
      cnt++;
    }
    return cnt;
  }
};
template <class R>
__device__ __forceinline__ int axis_stencil(double x, float dxf, double inv, int n, int wrap, int spread, int node[5],
                                            int*, R w[5]) {
  return Stencil<R>::axis(x, dxf, inv, n, wrap, spread, node, w);
}

// One marker's force onto its stencil nodes (global atomics).
template <class R>
__device__ __forceinline__ void spread_one(const LatticeConst& lk, R4<R>* Fc, double x, double y, double z, R Fx,
                                           R Fy, R Fz) {
  int nxa[5], nya[5], nza[5], rx[5], ry[5], rz[5];
  R wx[5], wy[5], wz[5];
  const int cxn = axis_stencil<R>(x, lk.dxf, lk.inv_dx, lk.nx, lk.ibm_wrap[0], 1, nxa, rx, wx);
  const int cyn = axis_stencil<R>(y, lk.dxf, lk.inv_dx, lk.ny, lk.ibm_wrap[1], 1, nya, ry, wy);
  const int czn = axis_stencil<R>(z, lk.dxf, lk.inv_dx, lk.nz, 0, 1, nza, rz, wz);
  for (int c = 0; c < czn; ++c)
    for (int b = 0; b < cyn; ++b)
      for (int a = 0; a < cxn; ++a) {
        const R delta = wx[a] * wy[b] * wz[c];
        const size_t n = (size_t)nxa[a] + (size_t)lk.nx * ((size_t)nya[b] + (size_t)lk.ny * nza[c]);
        atomic_add3(Fc, n, Fx * delta, Fy * delta, Fz * delta);
      }
}
// Lattice velocity (u/C) interpolated at one marker from the moments buffer.
template <class R>
__device__ __forceinline__ void interp_one(const LatticeConst& lk, const R4<R>* ubuf, double x, double y, double z,
                                           R& ax, R& ay, R& az) {
  int nxa[5], nya[5], nza[5], rx[5], ry[5], rz[5];
  R wx[5], wy[5], wz[5];
  const int cxn = axis_stencil<R>(x, lk.dxf, lk.inv_dx, lk.nx, lk.ibm_wrap[0], 0, nxa, rx, wx);
  const int cyn = axis_stencil<R>(y, lk.dxf, lk.inv_dx, lk.ny, lk.ibm_wrap[1], 0, nya, ry, wy);
  const int czn = axis_stencil<R>(z, lk.dxf, lk.inv_dx, lk.nz, 0, 0, nza, rz, wz);
  ax = 0; ay = 0; az = 0;
  for (int c = 0; c < czn; ++c)
    for (int b = 0; b < cyn; ++b)
      for (int a = 0; a < cxn; ++a) {
        const R delta = wx[a] * wy[b] * wz[c];
        const size_t n = (size_t)nxa[a] + (size_t)lk.nx * ((size_t)nya[b] + (size_t)lk.ny * nza[c]);
        const R4<R> u = ubuf[n];
        ax += u.y * delta; ay += u.z * delta; az += u.w * delta;
      }
}

// FP32 stencil as four fixed slots per axis (base + {-1..2}): a slot the
// variable-length stencil leaves out has weight zero and a clamped in-range
// node, so the fully unrolled 4x4x4 gather issues all 64 loads at once and
// adds the same non-zero terms in the same order (a zero term leaves a float
// sum unchanged).
__device__ __forceinline__ void axis_slot(int base, float fr, int n, int wrap, int s, int& node, float& w) {
  const float dd = fr - (float)(s - 1);
  float ws = fabsf(dd) < 2.f ? 0.25f * (1.f + cospif(0.5f * dd)) : 0.f;
  int nd = base + s - 1;
  if (nd < 0 || nd >= n) {
    if (wrap) {
      nd = wrapi(nd, n);
    } else {
      nd = nd < 0 ? 0 : n - 1;
      ws = 0.f;
    }
  }
  node = nd;
  w = ws;
}
__device__ __forceinline__ void axis_base(double x, double inv_dx, int& base, float& fr) {
  const double r = x * inv_dx;
  const double fb = floor(r);
  base = (int)fb;
  fr = (float)(r - fb);
}
__device__ __forceinline__ void axis4(double x, double inv_dx, int n, int wrap, int node[4], float w[4]) {
  int base;
  float fr;
  axis_base(x, inv_dx, base, fr);
#pragma unroll
  for (int s = 0; s < 4; ++s) axis_slot(base, fr, n, wrap, s, node[s], w[s]);
}
template <>
__device__ __forceinline__ void spread_one<float>(const LatticeConst& lk, R4<float>* Fc, double x, double y,
                                                  double z, float Fx, float Fy, float Fz) {
  int nxa[4], nya[4], nza[4];
  float wx[4], wy[4], wz[4];
  const double inv = lk.inv_dx;
  axis4(x, inv, lk.nx, lk.ibm_wrap[0], nxa, wx);
  axis4(y, inv, lk.ny, lk.ibm_wrap[1], nya, wy);
  axis4(z, inv, lk.nz, 0, nza, wz);
#pragma unroll
  for (int c = 0; c < 4; ++c)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const size_t row = (size_t)lk.nx * ((size_t)nya[b] + (size_t)lk.ny * nza[c]);
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        const float delta = wx[a] * wy[b] * wz[c];
        if (delta != 0.f) atomic_add3(Fc, row + nxa[a], Fx * delta, Fy * delta, Fz * delta);
      }
    }
}
template <>
__device__ __forceinline__ void interp_one<float>(const LatticeConst& lk, const R4<float>* ubuf, double x, double y,
                                                  double z, float& ax, float& ay, float& az) {
  int nxa[4], nya[4], nza[4];
  float wx[4], wy[4], wz[4];
  const double inv = lk.inv_dx;
  axis4(x, inv, lk.nx, lk.ibm_wrap[0], nxa, wx);
  axis4(y, inv, lk.ny, lk.ibm_wrap[1], nya, wy);
  axis4(z, inv, lk.nz, 0, nza, wz);
  ax = 0.f; ay = 0.f; az = 0.f;
#pragma unroll
  for (int c = 0; c < 4; ++c)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const size_t row = (size_t)lk.nx * ((size_t)nya[b] + (size_t)lk.ny * nza[c]);
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        const float delta = wx[a] * wy[b] * wz[c];
        // read-only within the kernel: through the non-coherent path
        // (interpolation 24.0 -> 21.0 us on the 256x128x128 channel)
        const R4<float> u = __ldg(ubuf + row + nxa[a]);
        ax += u.y * delta; ay += u.z * delta; az += u.w * delta;
      }
    }
}

// ---------------------------------------------------------------- spreading
// One thread per marker: total element force (membrane + Morse + bonds, kept
// for the element output) or fibrin force, onto the current force buffer.
template <class R>
__global__ void __launch_bounds__(128) spread_k(LatticeConst lk, R4<R>* FA, R4<R>* FB, int PE, const double* X,
                                                const double* Y, const double* Z, const R* Fmem,
                                                const double* Fmorse, const R* Fbond, double* Ftot, int M,
                                                const double* fX, const double* fY, const double* fZ,
                                                const double* fF, double F0, Control* ctl) {
  if (ctl->done) return;
  R4<R>* Fc = (ctl->step & 1) ? FB : FA;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  double x, y, z, fx, fy, fz;
  if (idx < PE) {
    x = X[idx]; y = Y[idx]; z = Z[idx];
    fx = (double)Fmem[idx]; fy = (double)Fmem[PE + idx]; fz = (double)Fmem[2 * PE + idx];
    if (Fmorse) { fx += Fmorse[idx]; fy += Fmorse[PE + idx]; fz += Fmorse[2 * PE + idx]; }
    if (Fbond) { fx += (double)Fbond[idx]; fy += (double)Fbond[PE + idx]; fz += (double)Fbond[2 * PE + idx]; }
    Ftot[idx] = fx; Ftot[PE + idx] = fy; Ftot[2 * PE + idx] = fz;
  } else if (idx < PE + M) {
    const int m = idx - PE;
    x = fX[m]; y = fY[m]; z = fZ[m];
    fx = fF[m] / F0; fy = fF[M + m] / F0; fz = fF[2 * M + m] / F0;
  } else {
    return;
  }
  spread_one<R>(lk, Fc, x, y, z, (R)fx, (R)fy, (R)fz);
}

// FP32 spreading of one force part as soon as it exists: n markers at
// (X, Y, Z) with force Fa (float, may be null) + Fd * rdiv (double, may be
// null), components n apart; markers whose part is zero add nothing.
__device__ __forceinline__ void spread_part_k_body(const LatticeConst& lk, float4* FA, float4* FB, int n,
                                                     const double* X, const double* Y, const double* Z,
                                                     const float* Fa, const double* Fd, double rdiv, Control* ctl, int bid, int nblk) {
  if (ctl->done) return;
  const int i = bid * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double fx = 0, fy = 0, fz = 0;
  if (Fa) { fx = (double)Fa[i]; fy = (double)Fa[n + i]; fz = (double)Fa[2 * n + i]; }
  // rdiv: 1/F0 for fibrin forces, formed once by the caller (FP64 division
  // is slow on this GPU)
  if (Fd) { fx += Fd[i] * rdiv; fy += Fd[n + i] * rdiv; fz += Fd[2 * n + i] * rdiv; }
  if (fx == 0 && fy == 0 && fz == 0) return;
  spread_one<float>(lk, (ctl->step & 1) ? FB : FA, X[i], Y[i], Z[i], (float)fx, (float)fy, (float)fz);
}
__global__ void __launch_bounds__(128) spread_part_k(LatticeConst lk, float4* FA, float4* FB, int n,
                                                     const double* X, const double* Y, const double* Z,
                                                     const float* Fa, const double* Fd, double rdiv, Control* ctl) {
  spread_part_k_body(lk, FA, FB, n, X, Y, Z, Fa, Fd, rdiv, ctl, blockIdx.x, gridDim.x);
}

// The same spreading with four lanes per marker: lane a of a marker's group
// takes the stencil's x slot a, so the 32 atomics of one warp instruction
// fall on 8 markers x 4 consecutive nodes (16 sectors of 32 bytes) instead
// of 32 scattered nodes.  The FP64 work is done once per marker (FP64 issues
// at a small fraction of the FP32 rate on this GPU): lane l < 3 forms force
// component l and the stencil base of axis l and the group shares them by
// shuffles.  Each node receives the same product as from spread_one; only
// the order of the atomic additions changes.  rdiv: the reciprocal of the
// divisor of Fd (1/F0 for fibrin forces), formed once by the caller.
constexpr int kSpreadLanes = 4;
__device__ __forceinline__ void spread4_body(const LatticeConst& lk, float4* FA, float4* FB, int n,
                                             const double* X, const double* Y, const double* Z, const float* Fa,
                                             const double* Fd, double rdiv, Control* ctl, int bid) {
  if (ctl->done) return;
  const long long t = (long long)bid * blockDim.x + threadIdx.x;
  const int i = (int)(t / kSpreadLanes), a = (int)(t % kSpreadLanes);
  const bool in = i < n;
  // groups are whole: every lane of an active group is in `act`
  const unsigned act = __ballot_sync(0xffffffffu, in);
  if (!in) return;
  const int l = a < 3 ? a : 2;
  double f = 0;
  if (Fa) f = (double)Fa[(size_t)l * n + i];
  if (Fd) f += Fd[(size_t)l * n + i] * rdiv;
  int base;
  float fr;
  axis_base(l == 0 ? X[i] : (l == 1 ? Y[i] : Z[i]), lk.inv_dx, base, fr);
  const unsigned nz = __ballot_sync(act, f != 0);
  const int g0 = (int)(threadIdx.x & 31u) & ~(kSpreadLanes - 1);
  const float fl = (float)f;
  const float Fx = __shfl_sync(act, fl, g0), Fy = __shfl_sync(act, fl, g0 + 1), Fz = __shfl_sync(act, fl, g0 + 2);
  const int bx = __shfl_sync(act, base, g0), by = __shfl_sync(act, base, g0 + 1), bz = __shfl_sync(act, base, g0 + 2);
  const float frx = __shfl_sync(act, fr, g0), fry = __shfl_sync(act, fr, g0 + 1), frz = __shfl_sync(act, fr, g0 + 2);
  if (((nz >> g0) & 7u) == 0u) return;  // no force in this part: nothing to add
  float4* Fc = (ctl->step & 1) ? FB : FA;
  int nxa;
  float wxa;
  axis_slot(bx, frx, lk.nx, lk.ibm_wrap[0], a, nxa, wxa);
  if (wxa == 0.f) return;
  int nya[4], nza[4];
  float wy[4], wz[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    axis_slot(by, fry, lk.ny, lk.ibm_wrap[1], q, nya[q], wy[q]);
    axis_slot(bz, frz, lk.nz, 0, q, nza[q], wz[q]);
  }
#pragma unroll
  for (int c = 0; c < 4; ++c)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const size_t row = (size_t)lk.nx * ((size_t)nya[b] + (size_t)lk.ny * nza[c]);
      const float delta = wxa * wy[b] * wz[c];
      if (delta != 0.f) atomic_add3(Fc, row + nxa, Fx * delta, Fy * delta, Fz * delta);
    }
}
__global__ void __launch_bounds__(128) spread4_k(LatticeConst lk, float4* FA, float4* FB, int n, const double* X,
                                                 const double* Y, const double* Z, const float* Fa,
                                                 const double* Fd, double rdiv, Control* ctl) {
  spread4_body(lk, FA, FB, n, X, Y, Z, Fa, Fd, rdiv, ctl, blockIdx.x);
}

// Force bricks of this step: every brick holding a lattice node that the
// spreading and interpolation stencils of a marker touch: base + {-2..2} per
// axis in FP64, base + {-1..2} in FP32, the base node being floor(x/dx) as
// the FP64 stencils form it, floor(x * (1/dx)) as the FP32 stencil does.
// Set before any force of the step exists, so the lattice pass over the
// other bricks can run while the forces are computed.  One bit per node (a
// brick is one 32-bit word): the position update sets each marker's bit for
// the next step, the bits are dilated in x, y and z by the stencil's reach
// (a mark at node b flags b-2 .. b+2 in FP64, b-1 .. b+2 in FP32); a
// non-zero word flags and lists its brick.
constexpr int kFlagR = 2;

// Sets the occupancy bit of a marker's base node; nodes outside the lattice
// are wrapped on IBM-periodic axes, else clamped to the face (its kFlagR
// neighbourhood still covers every in-range node the stencil can reach).
__device__ __forceinline__ void mark_node(const LatticeConst& lk, unsigned* mark, double x, double y, double z,
                                          bool fp64) {
  const double dxd = (double)lk.dxf, inv = lk.inv_dx;
  auto node = [&](double v, int n, int wrap) {
    // floor and conversion in one saturating instruction (NaN: 0), then
    // within +-1e9 so that the index arithmetic below cannot overflow
    int i = __double2int_rd(fp64 ? v / dxd : v * inv);
    i = i < -1000000000 ? -1000000000 : (i > 1000000000 ? 1000000000 : i);
    if (wrap) return wrapi(i, n);
    return i < 0 ? 0 : (i >= n ? n - 1 : i);
  };
  const int ix = node(x, lk.nx, lk.ibm_wrap[0]);
  const int iy = node(y, lk.ny, lk.ibm_wrap[1]);
  const int iz = node(z, lk.nz, 0);
  atomicOr(mark + (ix >> 5) + lk.nbx * (iy + lk.ny * iz), 1u << (ix & 31));
}

// occupancy of the initial positions (afterwards the position update marks
// the positions of the next step)
__global__ void __launch_bounds__(128) mark_markers_k(LatticeConst lk, unsigned* mark, int PE, const double* X,
                                                      const double* Y, const double* Z, int M, const double* fX,
                                                      const double* fY, const double* fZ, bool fp64) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < PE) mark_node(lk, mark, X[idx], Y[idx], Z[idx], fp64);
  else if (idx < PE + M) mark_node(lk, mark, fX[idx - PE], fY[idx - PE], fZ[idx - PE], fp64);
}

// word bx (C) of a row dilated by kFlagR bits in x, from its left and right
// neighbour words (periodic rows: across the row's ends; when nx is not a
// multiple of 32, a word next to occupied bits across the wrap is taken as
// all set, a superset)
// hi: reach of a mark towards lower x (nodes n - hi .. n flag from a mark at
// n, the stencil's upper reach); marks reach kFlagR nodes towards higher x.
__device__ __forceinline__ unsigned dilate_words(unsigned C, unsigned Lw, unsigned Rw, int bx, int nbx, bool wrap,
                                                 bool partial, int hi) {
  // a partial last word is not bit-adjacent to word 0 across the wrap
  if (partial && wrap && ((bx == 0 && Lw) || (bx == nbx - 1 && Rw))) return 0xffffffffu;
  if (!(C | Lw | Rw)) return 0u;
  const unsigned long long lo = ((unsigned long long)C << 32) | Lw;  // C above its left neighbour
  const unsigned long long hi_w = ((unsigned long long)Rw << 32) | C;  // C below its right neighbour
  unsigned long long dl = lo, dh = hi_w;
#pragma unroll
  for (int r = 1; r <= kFlagR; ++r) {
    dl |= lo << r;
    if (r <= hi) dh |= hi_w >> r;
  }
  return (unsigned)(dl >> 32) | (unsigned)dh;
}

// One kernel per step: each brick word dilated by the stencil's reach in x
// (bits), y (rows, wrapped on an IBM-periodic axis) and z (planes): marks up
// to kFlagR nodes below a node and up to hi above it (2 FP64, 1 FP32) flag
// it; a non-zero word flags and lists its brick (list[par],
// active_count[par]).  The dilation distributes over OR, so it is done
// separably: a CTA takes flag_rows() whole rows of one z-plane, ORs each row
// word (and its y halo) over the planes into shared memory, then over the
// rows, then dilates in x.
// The occupancy bits of the step (buffer par) are left for the
// flagged-brick lattice pass to clear.  With the near region of the
// pipelined schedule (nearA/B): a flagged brick outside it was updated
// without force by the far pass, an error (a marker moved more than one
// node in one step).
constexpr int kFlagThreads = 256;
constexpr int kFlagWords = 4096;  // shared words per stage (rows + halo) x nbx
__host__ __device__ inline int flag_rows(int nbx) {
  int r = kFlagThreads / nbx;
  if (r < 1) r = 1;
  while (r > 1 && (r + 2 * kFlagR) * nbx > kFlagWords) --r;
  return r;
}
__device__ __forceinline__ void flag_k_body(const LatticeConst& lk, const unsigned* mark, unsigned* flA,
                                                       unsigned* flB, int* lA, int* lB, const unsigned char* nearA,
                                                       const unsigned char* nearB, int hi, Control* ctl, int bid, int nblk,
                                                       bool with_prev = false) {
  if (ctl->done) return;
  __shared__ unsigned s_z[kFlagWords];  // OR over the planes, rows y0-2 .. y0+R+1
  __shared__ unsigned s_yz[kFlagWords];  // OR over the rows too, rows y0 .. y0+R-1
  const int par = (int)(ctl->step & 1);
  const unsigned* mk = mark + (size_t)par * lk.nbricks;
  unsigned* fl = par ? flB : flA;
  const unsigned* flprev = par ? flA : flB;  // the previous step's flags
  int* list = par ? lB : lA;
  const unsigned char* nr = par ? nearB : nearA;
  const int lane = threadIdx.x & 31;
  const bool wrap = lk.ibm_wrap[0] != 0, partial = (lk.nx & 31) != 0;
  const int nbx = lk.nbx, R = flag_rows(nbx);
  const int ytiles = (lk.ny + R - 1) / R;
  const int z = bid / ytiles, y0 = (bid % ytiles) * R;
  const int halo = (R + 2 * kFlagR) * nbx;
  for (int i = threadIdx.x; i < halo; i += kFlagThreads) {
    const int bx = i % nbx;
    int yy = y0 - kFlagR + i / nbx;
    unsigned acc = 0;
    bool ok = true;
    if (yy < 0 || yy >= lk.ny) {
      ok = lk.ibm_wrap[1] != 0;
      yy = wrapi(yy, lk.ny);
    }
    if (ok)
#pragma unroll
      for (int dz = -kFlagR; dz <= kFlagR; ++dz) {
        if (dz > hi) break;
        const int zz = z + dz;
        if (zz >= 0 && zz < lk.nz) acc |= mk[bx + (size_t)nbx * (yy + (size_t)lk.ny * zz)];
      }
    s_z[i] = acc;
  }
  __syncthreads();
  const int outs = R * nbx;
  for (int i = threadIdx.x; i < outs; i += kFlagThreads) {
    unsigned acc = 0;
#pragma unroll
    for (int dy = 0; dy <= 2 * kFlagR; ++dy)
      if (dy <= kFlagR + hi) acc |= s_z[i + dy * nbx];
    s_yz[i] = acc;
  }
  __syncthreads();
  // rounds of kFlagThreads so that every lane of a warp reaches the ballot
  for (int i0 = 0; i0 < outs; i0 += kFlagThreads) {
    const int i = i0 + threadIdx.x;
    const int bx = i % nbx, y = y0 + i / nbx;
    bool f = false, listed = false;
    int w = 0;
    if (i < outs && y < lk.ny) {
      const int rowbase = i - bx;
      const unsigned C = s_yz[i];
      const unsigned Lw = bx > 0 ? s_yz[i - 1] : (wrap ? s_yz[rowbase + nbx - 1] : 0u);
      const unsigned Rw = bx < nbx - 1 ? s_yz[i + 1] : (wrap ? s_yz[rowbase] : 0u);
      w = bx + nbx * (y + lk.ny * z);
      f = dilate_words(C, Lw, Rw, bx, nbx, wrap, partial, hi) != 0u;
      if (f) {
        fl[w] = 1u;
        if (nr && !nr[w]) atomicOr(&ctl->err, ERR_FAR_FLAGGED);
      }
      // with_prev: the flagged-brick pass also takes the bricks that had a
      // force in the previous step (the quiet pass leaves them out)
      listed = f || (with_prev && flprev[w] != 0u);
    }
    const unsigned bal = __ballot_sync(0xffffffffu, listed);
    if (bal) {
      int base = 0;
      if (lane == 0) base = atomicAdd(&ctl->active_count[par], __popc(bal));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (listed) list[base + __popc(bal & ((1u << lane) - 1u))] = w;
    }
  }
}
__global__ void __launch_bounds__(kFlagThreads) flag_k(LatticeConst lk, const unsigned* mark, unsigned* flA,
                                                       unsigned* flB, int* lA, int* lB, const unsigned char* nearA,
                                                       const unsigned char* nearB, int hi, Control* ctl,
                                                       bool with_prev) {
  flag_k_body(lk, mark, flA, flB, lA, lB, nearA, nearB, hi, ctl, blockIdx.x, gridDim.x, with_prev);
}

// ------------------------------------------------------- interp + advance
// Morse cell of a position and the position relative to the cell's corner
// (periodic axes wrapped first), the same rule as the oracle's cell list.
__device__ __forceinline__ int cell_of(const PlateletConst& k, double x, double y, double z, float rel[3] = nullptr,
                                       int cc[3] = nullptr) {
  const double p[3] = {x, y, z};
  int c[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    double v = p[a];
    if (k.wrap[a]) v -= k.L[a] * floor(v / k.L[a]);
    int ci = (int)floor(v / k.cs[a]);
    if (ci < 0) ci = 0;
    if (ci >= k.ncell[a]) ci = k.ncell[a] - 1;
    c[a] = ci;
    if (rel) rel[a] = (float)(v - ci * k.cs[a]);
    if (cc) cc[a] = ci;
  }
  return c[0] + k.ncell[0] * (c[1] + k.ncell[1] * c[2]);
}
__device__ __forceinline__ void bin_put(const PlateletConst& k, double x, double y, double z, int g, int* bin_count,
                                        float4* bin, Control* ctl) {
  float rel[3];
  const int c = cell_of(k, x, y, z, rel);
  const int slot = atomicAdd(bin_count + c, 1);
  // the first element of a cell lists the cell as occupied (the list sits
  // after the bins: occupied[ncells])
  if (slot == 0) {
    int* occ = reinterpret_cast<int*>(bin + (size_t)k.ncell[0] * k.ncell[1] * k.ncell[2] * kBinCap);
    occ[atomicAdd(&ctl->occupied, 1)] = c;
  }
  if (slot < kBinCap) bin[(size_t)c * kBinCap + slot] = make_float4(rel[0], rel[1], rel[2], __int_as_float(g));
  else atomicOr(&ctl->err, ERR_BIN_OVERFLOW);
}

// Position update of marker idx (element idx < PE, else fibrin node idx-PE)
// with its interpolated lattice velocity (lattice units): velocity store,
// move (fixed fibrin nodes stay), periodic wrap, Morse binning, occupancy
// bit of the next step.
__device__ __forceinline__ void advance_marker(const LatticeConst& lk, const PlateletConst& pk, int idx, int PE,
                                               double x, double y, double z, double ax, double ay, double az,
                                               double* X, double* Y, double* RY, double* Z, double* V, int M,
                                               double* fX, double* fY, double* fZ, double* fV, const int* ffix,
                                               int* bin_count, float4* bin, unsigned* mark, Control* ctl,
                                               bool fp64) {
  const double vx = ax * lk.C, vy = ay * lk.C, vz = az * lk.C;
  const float dtT = lk.dtT;
  const double Lx = lk.Lx, Ly = lk.Ly;
  if (idx < PE) {
    V[idx] = vx; V[PE + idx] = vy; V[2 * PE + idx] = vz;
    x += vx * dtT;
    if (lk.ibm_wrap[0]) { if (x > Lx) x -= Lx; else if (x < 0) x += Lx; }
    y += vy * dtT;
    if (lk.ibm_wrap[1]) { if (y > Ly) y -= Ly; else if (y < 0) y += Ly; }
    RY[idx] += vy * dtT;
    z += vz * dtT;
    X[idx] = x; Y[idx] = y; Z[idx] = z;
    if (bin) bin_put(pk, x, y, z, idx, bin_count, bin, ctl);
  } else {
    const int m = idx - PE;
    fV[m] = vx; fV[M + m] = vy; fV[2 * M + m] = vz;
    if (!ffix[m]) {
      x += vx * dtT;
      if (lk.ibm_wrap[0]) { if (x > Lx) x -= Lx; else if (x < 0) x += Lx; }
      y += vy * dtT;
      if (lk.ibm_wrap[1]) { if (y > Ly) y -= Ly; else if (y < 0) y += Ly; }
      z += vz * dtT;
      fX[m] = x; fY[m] = y; fZ[m] = z;
    }
  }
  // the occupancy bits of the next step (buffer of the other parity)
  mark_node(lk, mark + (size_t)((int)(ctl->step & 1) ^ 1) * lk.nbricks, x, y, z, fp64);
}

// The last block to finish closes the step: counter, first flag, the other
// force buffer's list, and the detach test of the next step
// (semLB.cu:451-455).
__device__ __forceinline__ void close_step(const PlateletConst& pk, Control* ctl, unsigned* done_blocks,
                                           double detach_rate, uint64_t seed, int nblk) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(done_blocks, 1u);
    if (prev == (unsigned)nblk - 1) {
      __threadfence();
      // the next step flags into the other force buffer: empty its list
      ctl->active_count[(int)(ctl->step & 1) ^ 1] = 0;
      const long long s = ctl->step + 1;
      ctl->step = s;
      ctl->first = 0;
      // a platelet without receptors has no bonds (the reference's bond
      // kernel then runs with no threads and totalBond stays at zero)
      if (!pk.nrec || !pk.P) ctl->total_bond = 0;
      if (detach_rate > 0 && ctl->total_bond == 0 && detach_uniform(seed, s) < detach_rate) ctl->done = 1;
      if (!ctl->done && ctl->stop > 0 && s >= ctl->stop) ctl->done = 2;
      *done_blocks = 0u;
    }
  }
}

// Ftot (optional): the element force total of the step (membrane + Morse +
// bonds), written here when the parts were spread separately.
template <class R>
__device__ __forceinline__ void interp_advance_k_body(const LatticeConst& lk, const PlateletConst& pk, const R4<R>* ubuf,
                                                        int PE, double* X, double* Y, double* RY, double* Z,
                                                        double* V, int M, double* fX, double* fY, double* fZ,
                                                        double* fV, const int* ffix, int* bin_count, float4* bin,
                                                        unsigned* mark, Control* ctl, unsigned* done_blocks,
                                                        double detach_rate, uint64_t seed, const R* Fmem,
                                                        const double* Fmorse, const R* Fbond, double* Ftot, int bid, int nblk) {
  if (ctl->done) return;
  const int idx = bid * blockDim.x + threadIdx.x;
  if (idx < PE + M) {
    const bool el = idx < PE;
    const int m = idx - PE;
    if (el && Ftot) {
      double fx = (double)Fmem[idx], fy = (double)Fmem[PE + idx], fz = (double)Fmem[2 * PE + idx];
      if (Fmorse) { fx += Fmorse[idx]; fy += Fmorse[PE + idx]; fz += Fmorse[2 * PE + idx]; }
      if (Fbond) { fx += (double)Fbond[idx]; fy += (double)Fbond[PE + idx]; fz += (double)Fbond[2 * PE + idx]; }
      Ftot[idx] = fx; Ftot[PE + idx] = fy; Ftot[2 * PE + idx] = fz;
    }
    const double x = el ? X[idx] : fX[m], y = el ? Y[idx] : fY[m], z = el ? Z[idx] : fZ[m];
    R ax, ay, az;
    interp_one<R>(lk, ubuf, x, y, z, ax, ay, az);
    advance_marker(lk, pk, idx, PE, x, y, z, (double)ax, (double)ay, (double)az, X, Y, RY, Z, V, M, fX, fY, fZ,
                   fV, ffix, bin_count, bin, mark, ctl, sizeof(R) == 8);
  }
  close_step(pk, ctl, done_blocks, detach_rate, seed, nblk);
}
template <class R>
__global__ void __launch_bounds__(128) interp_advance_k(LatticeConst lk, PlateletConst pk, const R4<R>* ubuf,
                                                        int PE, double* X, double* Y, double* RY, double* Z,
                                                        double* V, int M, double* fX, double* fY, double* fZ,
                                                        double* fV, const int* ffix, int* bin_count, float4* bin,
                                                        unsigned* mark, Control* ctl, unsigned* done_blocks,
                                                        double detach_rate, uint64_t seed, const R* Fmem,
                                                        const double* Fmorse, const R* Fbond, double* Ftot) {
  interp_advance_k_body<R>(lk, pk, ubuf, PE, X, Y, RY, Z, V, M, fX, fY, fZ, fV, ffix, bin_count, bin, mark, ctl, done_blocks, detach_rate, seed, Fmem, Fmorse, Fbond, Ftot, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------ platelet boxes (FP32)
// FP32 spreading and interpolation of platelet elements through a per-platelet
// box of lattice nodes in shared memory: one CTA per platelet; the box spans
// the FP32 stencils (base node + {-1..2} per axis) of all its elements, node
// indices taken relative to the first element's base node (minimum image on
// periodic axes).  Weights and nodes are those of the per-marker kernels;
// only the order of the float sums differs.  A platelet whose box exceeds
// kBoxCap nodes, and every fibrin node, takes the per-marker path.
constexpr int kBoxThreads = 512;
constexpr int kBoxCap = 8192;    // nodes of a platelet box
constexpr int kBoxElems = 1024;  // elements of a platelet staged in shared memory
constexpr int kBoxFibrin = 128;  // fibrin nodes per CTA of the box kernels

struct BoxAxis {
  int base;  // node floor(x / dx)
  float fr;  // x / dx - base
};
__device__ __forceinline__ BoxAxis box_axis(double x, double inv) {
  const double r = x * inv;
  const double fb = floor(r);
  return BoxAxis{(int)fb, (float)(r - fb)};
}
// weight of stencil offset o (the FP32 stencil's rule); false outside the
// support
__device__ __forceinline__ bool box_weight(float fr, int o, float& w) {
  const float dd = fr - (float)o;
  if (!(fabsf(dd) < 2.f)) return false;
  w = 0.25f * (1.f + cospif(0.5f * dd));
  return true;
}

// Box geometry of a platelet from its elements' base nodes SB[axis][0..E)
// (stride kBoxElems); returns false (box too large, or non-finite
// positions) for the per-marker path.  i0: first element's base node;
// lo/ext: box origin (relative to i0) and extent per axis.
__device__ bool platelet_box(const LatticeConst& lk, const int* SB, int E, int i0[3], int lo[3], int ext[3]) {
  __shared__ int s_min[3], s_max[3];
  const int n3[3] = {lk.nx, lk.ny, lk.nz};
  const int wrap3[3] = {lk.ibm_wrap[0], lk.ibm_wrap[1], 0};
#pragma unroll
  for (int a = 0; a < 3; ++a) i0[a] = SB[a * kBoxElems];
  if (threadIdx.x < 3) { s_min[threadIdx.x] = 0x7fffffff; s_max[threadIdx.x] = -0x7fffffff; }
  __syncthreads();
  int mn[3] = {0x7fffffff, 0x7fffffff, 0x7fffffff}, mx[3] = {-0x7fffffff, -0x7fffffff, -0x7fffffff};
  for (int e = threadIdx.x; e < E; e += blockDim.x) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      int d = SB[a * kBoxElems + e] - i0[a];
      if (wrap3[a]) d = wrapi(d + n3[a] / 2, n3[a]) - n3[a] / 2;
      mn[a] = min(mn[a], d);
      mx[a] = max(mx[a], d);
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    atomicMin(&s_min[a], mn[a]);
    atomicMax(&s_max[a], mx[a]);
  }
  __syncthreads();
  long long vol = 1;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const long long e = (long long)s_max[a] - (long long)s_min[a] + 4;
    if (e <= 0 || e > kBoxCap) return false;  // also non-finite positions
    lo[a] = s_min[a] - 1;
    ext[a] = (int)e;
    vol *= e;
  }
  return vol <= kBoxCap;
}

// Stages element e's base node and fraction per axis (FP64 to lattice
// units once per element; the warp loops then use only these).
__device__ __forceinline__ void stage_element(int* SB, float* SF, int e, double x, double y, double z, double inv) {
  const double p3[3] = {x, y, z};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const BoxAxis ba = box_axis(p3[a], inv);
    SB[a * kBoxElems + e] = ba.base;
    SF[a * kBoxElems + e] = ba.fr;
  }
}

// global node of box offset d (relative to i0) on one axis; -1 if outside a
// non-periodic lattice
__device__ __forceinline__ int box_global(int i0, int d, int n, int wrap) {
  const int g = i0 + d;
  if (g >= 0 && g < n) return g;
  return wrap ? wrapi(g, n) : -1;
}

// Shared-memory layout of the box kernels: the node box [3][kBoxCap] floats,
// then per element (stride kBoxElems) its position (3 doubles), base node
// (3 ints), fraction (3 floats) and a float3 (force or velocity).
constexpr size_t kBoxSmem =
    3 * kBoxCap * sizeof(float) + (size_t)kBoxElems * (3 * sizeof(double) + 3 * sizeof(int) + 6 * sizeof(float));

__global__ void __launch_bounds__(kBoxThreads) spread_box_k(LatticeConst lk, float4* FA, float4* FB, int P, int E,
                                                            const double* X, const double* Y, const double* Z,
                                                            const float* Fmem, const double* Fmorse,
                                                            const float* Fbond, double* Ftot, int M,
                                                            const double* fX, const double* fY, const double* fZ,
                                                            const double* fF, double F0, Control* ctl) {
  if (ctl->done) return;
  float4* Fc = (ctl->step & 1) ? FB : FA;
  const int PE = P * E;
  if ((int)blockIdx.x >= P) {
    // fibrin nodes: per-marker atomics, kBoxFibrin per CTA (spread over SMs)
    const int m = ((int)blockIdx.x - P) * kBoxFibrin + threadIdx.x;
    if (threadIdx.x < kBoxFibrin && m < M)
      spread_one<float>(lk, Fc, fX[m], fY[m], fZ[m], (float)(fF[m] / F0), (float)(fF[M + m] / F0),
                        (float)(fF[2 * M + m] / F0));
    return;
  }
  extern __shared__ __align__(16) unsigned char s_raw[];
  float* s_box = reinterpret_cast<float*>(s_raw);
  double* s_pos = reinterpret_cast<double*>(s_box + 3 * kBoxCap);  // [3][kBoxElems]
  float* s_f = reinterpret_cast<float*>(s_pos + 3 * kBoxElems);     // [3][kBoxElems]
  int* s_b = reinterpret_cast<int*>(s_f + 3 * kBoxElems);           // [3][kBoxElems] base nodes
  float* s_fr = reinterpret_cast<float*>(s_b + 3 * kBoxElems);      // [3][kBoxElems] fractions
  const int p = blockIdx.x, base = p * E;
  const bool staged = E <= kBoxElems;
  const double inv = lk.inv_dx;
  // element forces (kept for the element output) and positions, thread per
  // element
  for (int e = threadIdx.x; e < E; e += blockDim.x) {
    const int g = base + e;
    double fx = (double)Fmem[g], fy = (double)Fmem[PE + g], fz = (double)Fmem[2 * PE + g];
    if (Fmorse) { fx += Fmorse[g]; fy += Fmorse[PE + g]; fz += Fmorse[2 * PE + g]; }
    if (Fbond) { fx += (double)Fbond[g]; fy += (double)Fbond[PE + g]; fz += (double)Fbond[2 * PE + g]; }
    Ftot[g] = fx; Ftot[PE + g] = fy; Ftot[2 * PE + g] = fz;
    if (staged) {
      const double x = X[g], y = Y[g], z = Z[g];
      s_pos[e] = x; s_pos[kBoxElems + e] = y; s_pos[2 * kBoxElems + e] = z;
      stage_element(s_b, s_fr, e, x, y, z, inv);
      s_f[e] = (float)fx; s_f[kBoxElems + e] = (float)fy; s_f[2 * kBoxElems + e] = (float)fz;
    } else {
      spread_one<float>(lk, Fc, X[g], Y[g], Z[g], (float)fx, (float)fy, (float)fz);
    }
  }
  if (!staged) return;
  __syncthreads();
  int i0[3], lo[3], ext[3];
  if (!platelet_box(lk, s_b, E, i0, lo, ext)) {
    for (int e = threadIdx.x; e < E; e += blockDim.x)
      spread_one<float>(lk, Fc, s_pos[e], s_pos[kBoxElems + e], s_pos[2 * kBoxElems + e], s_f[e],
                        s_f[kBoxElems + e], s_f[2 * kBoxElems + e]);
    return;
  }
  const int vol = ext[0] * ext[1] * ext[2];
  for (int i = threadIdx.x; i < vol; i += blockDim.x) {
    s_box[i] = 0.f;
    s_box[kBoxCap + i] = 0.f;
    s_box[2 * kBoxCap + i] = 0.f;
  }
  __syncthreads();
  const int n3[3] = {lk.nx, lk.ny, lk.nz};
  const int wrap3[3] = {lk.ibm_wrap[0], lk.ibm_wrap[1], 0};
  // one warp per element, one lane per pair of its 4x4x4 stencil nodes
  // (x offset lane&3, y offset (lane>>2)&3, z offsets lane>>4 and +2): the
  // 64 shared-memory atomics of an element go to distinct nodes
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int oa = (lane & 3) - 1, ob = ((lane >> 2) & 3) - 1, oc = (lane >> 4) - 1;
  for (int e = warp; e < E; e += nwarps) {
    int dd[3];
    float fr[3];
#pragma unroll
    for (int ax3 = 0; ax3 < 3; ++ax3) {
      int d = s_b[ax3 * kBoxElems + e] - i0[ax3];
      if (wrap3[ax3]) d = wrapi(d + n3[ax3] / 2, n3[ax3]) - n3[ax3] / 2;
      dd[ax3] = d;
      fr[ax3] = s_fr[ax3 * kBoxElems + e];
    }
    float wx, wy;
    const bool okx = box_weight(fr[0], oa, wx) && box_global(i0[0], dd[0] + oa, n3[0], wrap3[0]) >= 0;
    const bool oky = box_weight(fr[1], ob, wy) && box_global(i0[1], dd[1] + ob, n3[1], wrap3[1]) >= 0;
    if (!(okx && oky)) continue;
    const float wxy = wx * wy;
    const float Fx = s_f[e], Fy = s_f[kBoxElems + e], Fz = s_f[2 * kBoxElems + e];
#pragma unroll
    for (int k2 = 0; k2 < 2; ++k2) {
      const int o = oc + 2 * k2;
      float wz;
      if (!(box_weight(fr[2], o, wz) && box_global(i0[2], dd[2] + o, n3[2], 0) >= 0)) continue;
      const float delta = wxy * wz;
      const int i = (dd[0] + oa - lo[0]) + ext[0] * ((dd[1] + ob - lo[1]) + ext[1] * (dd[2] + o - lo[2]));
      atomicAdd(&s_box[i], Fx * delta);
      atomicAdd(&s_box[kBoxCap + i], Fy * delta);
      atomicAdd(&s_box[2 * kBoxCap + i], Fz * delta);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < vol; i += blockDim.x) {
    const float vx = s_box[i], vy = s_box[kBoxCap + i], vz = s_box[2 * kBoxCap + i];
    if (vx == 0.f && vy == 0.f && vz == 0.f) continue;
    const int ax = i % ext[0], ay = (i / ext[0]) % ext[1], az = i / (ext[0] * ext[1]);
    const int gx = box_global(i0[0], lo[0] + ax, lk.nx, lk.ibm_wrap[0]);
    const int gy = box_global(i0[1], lo[1] + ay, lk.ny, lk.ibm_wrap[1]);
    const int gz = box_global(i0[2], lo[2] + az, lk.nz, 0);
    if (gx < 0 || gy < 0 || gz < 0) continue;
    atomicAdd(Fc + (size_t)gx + (size_t)lk.nx * ((size_t)gy + (size_t)lk.ny * gz), make_float4(vx, vy, vz, 0.f));
  }
}

__global__ void __launch_bounds__(kBoxThreads) interp_box_k(LatticeConst lk, PlateletConst pk, const float4* ubuf,
                                                            int P, int E, double* X, double* Y, double* RY,
                                                            double* Z, double* V, int M, double* fX, double* fY,
                                                            double* fZ, double* fV, const int* ffix, int* bin_count,
                                                            float4* bin, unsigned* mark, Control* ctl,
                                                            unsigned* done_blocks, double detach_rate,
                                                            uint64_t seed) {
  if (ctl->done) return;
  const int PE = P * E;
  if ((int)blockIdx.x >= P) {
    const int m = ((int)blockIdx.x - P) * kBoxFibrin + threadIdx.x;
    if (threadIdx.x < kBoxFibrin && m < M) {
      const double x = fX[m], y = fY[m], z = fZ[m];
      float ax, ay, az;
      interp_one<float>(lk, ubuf, x, y, z, ax, ay, az);
      advance_marker(lk, pk, PE + m, PE, x, y, z, (double)ax, (double)ay, (double)az, X, Y, RY, Z, V, M, fX, fY,
                     fZ, fV, ffix, bin_count, bin, mark, ctl, false);
    }
    close_step(pk, ctl, done_blocks, detach_rate, seed, gridDim.x);
    return;
  }
  extern __shared__ __align__(16) unsigned char s_raw[];
  float* s_box = reinterpret_cast<float*>(s_raw);                   // lattice velocity of the box nodes
  double* s_pos = reinterpret_cast<double*>(s_box + 3 * kBoxCap);  // [3][kBoxElems]
  float* s_v = reinterpret_cast<float*>(s_pos + 3 * kBoxElems);     // [3][kBoxElems] interpolated velocity
  int* s_b = reinterpret_cast<int*>(s_v + 3 * kBoxElems);           // [3][kBoxElems] base nodes
  float* s_fr = reinterpret_cast<float*>(s_b + 3 * kBoxElems);      // [3][kBoxElems] fractions
  const int p = blockIdx.x, base = p * E;
  const bool staged = E <= kBoxElems;
  const double inv = lk.inv_dx;
  if (!staged) {
    for (int e = threadIdx.x; e < E; e += blockDim.x) {
      const int g = base + e;
      const double x = X[g], y = Y[g], z = Z[g];
      float ax, ay, az;
      interp_one<float>(lk, ubuf, x, y, z, ax, ay, az);
      advance_marker(lk, pk, g, PE, x, y, z, (double)ax, (double)ay, (double)az, X, Y, RY, Z, V, M, fX, fY, fZ,
                     fV, ffix, bin_count, bin, mark, ctl, false);
    }
    close_step(pk, ctl, done_blocks, detach_rate, seed, gridDim.x);
    return;
  }
  for (int e = threadIdx.x; e < E; e += blockDim.x) {
    const double x = X[base + e], y = Y[base + e], z = Z[base + e];
    s_pos[e] = x;
    s_pos[kBoxElems + e] = y;
    s_pos[2 * kBoxElems + e] = z;
    stage_element(s_b, s_fr, e, x, y, z, inv);
  }
  __syncthreads();
  int i0[3], lo[3], ext[3];
  const bool boxed = platelet_box(lk, s_b, E, i0, lo, ext);
  if (boxed) {
    const int vol = ext[0] * ext[1] * ext[2];
    for (int i = threadIdx.x; i < vol; i += blockDim.x) {
      const int ax = i % ext[0], ay = (i / ext[0]) % ext[1], az = i / (ext[0] * ext[1]);
      const int gx = box_global(i0[0], lo[0] + ax, lk.nx, lk.ibm_wrap[0]);
      const int gy = box_global(i0[1], lo[1] + ay, lk.ny, lk.ibm_wrap[1]);
      const int gz = box_global(i0[2], lo[2] + az, lk.nz, 0);
      float4 u = make_float4(0.f, 0.f, 0.f, 0.f);
      if (gx >= 0 && gy >= 0 && gz >= 0) u = ubuf[(size_t)gx + (size_t)lk.nx * ((size_t)gy + (size_t)lk.ny * gz)];
      s_box[i] = u.y; s_box[kBoxCap + i] = u.z; s_box[2 * kBoxCap + i] = u.w;
    }
    __syncthreads();
    const int n3[3] = {lk.nx, lk.ny, lk.nz};
    const int wrap3[3] = {lk.ibm_wrap[0], lk.ibm_wrap[1], 0};
    // one warp per element, one lane per pair of its stencil nodes
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int oa = (lane & 3) - 1, ob = ((lane >> 2) & 3) - 1, oc = (lane >> 4) - 1;
    for (int e = warp; e < E; e += nwarps) {
      int dd[3];
      float fr[3];
#pragma unroll
      for (int ax3 = 0; ax3 < 3; ++ax3) {
        int d = s_b[ax3 * kBoxElems + e] - i0[ax3];
        if (wrap3[ax3]) d = wrapi(d + n3[ax3] / 2, n3[ax3]) - n3[ax3] / 2;
        dd[ax3] = d;
        fr[ax3] = s_fr[ax3 * kBoxElems + e];
      }
      float ax = 0.f, ay = 0.f, az = 0.f;
      float wx, wy;
      const bool okx = box_weight(fr[0], oa, wx) && box_global(i0[0], dd[0] + oa, n3[0], wrap3[0]) >= 0;
      const bool oky = box_weight(fr[1], ob, wy) && box_global(i0[1], dd[1] + ob, n3[1], wrap3[1]) >= 0;
      if (okx && oky) {
        const float wxy = wx * wy;
#pragma unroll
        for (int k2 = 0; k2 < 2; ++k2) {
          const int o = oc + 2 * k2;
          float wz;
          if (!(box_weight(fr[2], o, wz) && box_global(i0[2], dd[2] + o, n3[2], 0) >= 0)) continue;
          const float delta = wxy * wz;
          const int i = (dd[0] + oa - lo[0]) + ext[0] * ((dd[1] + ob - lo[1]) + ext[1] * (dd[2] + o - lo[2]));
          ax += s_box[i] * delta;
          ay += s_box[kBoxCap + i] * delta;
          az += s_box[2 * kBoxCap + i] * delta;
        }
      }
#pragma unroll
      for (int sh = 16; sh > 0; sh >>= 1) {
        ax += __shfl_xor_sync(0xffffffffu, ax, sh);
        ay += __shfl_xor_sync(0xffffffffu, ay, sh);
        az += __shfl_xor_sync(0xffffffffu, az, sh);
      }
      if (lane == 0) { s_v[e] = ax; s_v[kBoxElems + e] = ay; s_v[2 * kBoxElems + e] = az; }
    }
  } else {
    for (int e = threadIdx.x; e < E; e += blockDim.x) {
      float ax, ay, az;
      interp_one<float>(lk, ubuf, s_pos[e], s_pos[kBoxElems + e], s_pos[2 * kBoxElems + e], ax, ay, az);
      s_v[e] = ax; s_v[kBoxElems + e] = ay; s_v[2 * kBoxElems + e] = az;
    }
  }
  __syncthreads();
  // thread per element: move it
  for (int e = threadIdx.x; e < E; e += blockDim.x)
    advance_marker(lk, pk, base + e, PE, s_pos[e], s_pos[kBoxElems + e], s_pos[2 * kBoxElems + e], (double)s_v[e],
                   (double)s_v[kBoxElems + e], (double)s_v[2 * kBoxElems + e], X, Y, RY, Z, V, M, fX, fY, fZ, fV,
                   ffix, bin_count, bin, mark, ctl, false);
  close_step(pk, ctl, done_blocks, detach_rate, seed, gridDim.x);
}

__global__ void bin_elements_k(PlateletConst pk, int PE, const double* X, const double* Y, const double* Z,
                               int* bin_count, float4* bin, Control* ctl) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= PE) return;
  bin_put(pk, X[g], Y[g], Z[g], g, bin_count, bin, ctl);
}

// ---------------------------------------------------------------- membrane
// Gaussian elimination with partial pivoting on [3][4], normalising pivot
// rows (sem_kernel.cu:249-284), and the row solve of :286-311.
template <class R>
__device__ __forceinline__ void gauss34(R g[3][4]) {
  int i = 0, j = 0;
  while (i < 3 && j < 3) {
    int maxi = i;
    for (int k = i + 1; k < 3; ++k)
      if (fabs(g[k][j]) > fabs(g[maxi][j])) maxi = k;
    if (g[maxi][j] != 0) {
      R piv = 0;
      for (int k = j; k < 4; ++k) {
        R t = g[i][k];
        g[i][k] = g[maxi][k];
        g[maxi][k] = t;
        if (k == j) piv = g[i][j];
        g[i][k] /= piv;
      }
      for (int k = i + 1; k < 3; ++k) {
        R f = g[k][j];
        for (int l = j; l < 4; ++l) g[k][l] -= f * g[i][l];
      }
      i++;
    }
    j++;
  }
}

// The same elimination on [A | b1 b2 b3]: pivots depend on A only, so each
// right-hand side sees exactly the operations of a separate 3x4 solve.
template <class R>
__device__ __forceinline__ void gauss36(R g[3][6]) {
  int i = 0, j = 0;
  while (i < 3 && j < 3) {
    int maxi = i;
    for (int k = i + 1; k < 3; ++k)
      if (fabs(g[k][j]) > fabs(g[maxi][j])) maxi = k;
    if (g[maxi][j] != 0) {
      R piv = 0;
      for (int k = j; k < 6; ++k) {
        R t = g[i][k];
        g[i][k] = g[maxi][k];
        g[maxi][k] = t;
        if (k == j) piv = g[i][j];
        g[i][k] /= piv;
      }
      for (int k = i + 1; k < 3; ++k) {
        R f = g[k][j];
        for (int l = j; l < 6; ++l) g[k][l] -= f * g[i][l];
      }
      i++;
    }
    j++;
  }
}

template <class R>
__device__ __forceinline__ R nrm3(R a, R b, R c) {
  return sqrt(a * a + b * b + c * c);
}

// Derivatives of the quadratic 6-node triangle's shape functions at its
// node li, (s, t) = (0,0) (1,0) (0,1) (.5,0) (0,.5) (.5,.5):
// N0 = (1-s-t)(1-2s-2t), N1 = s(2s-1), N2 = t(2t-1), N3 = 4s(1-s-t),
// N4 = 4t(1-s-t), N5 = 4st (the table of sem_kernel.cu:92-100).
template <class R>
__device__ __forceinline__ void p2_grad(int li, R gs[6], R gt[6]) {
  const R s_ = (li == 1) ? (R)1 : (li == 3 || li == 5) ? (R)0.5 : (R)0;
  const R t_ = (li == 2) ? (R)1 : (li == 4 || li == 5) ? (R)0.5 : (R)0;
  gs[0] = 4 * s_ + 4 * t_ - 3; gs[1] = 4 * s_ - 1; gs[2] = 0;
  gs[3] = -8 * s_ - 4 * t_ + 4; gs[4] = -4 * t_; gs[5] = 4 * t_;
  gt[0] = 4 * t_ + 4 * s_ - 3; gt[1] = 0; gt[2] = 4 * t_ - 1;
  gt[3] = -4 * s_; gt[4] = -8 * t_ - 4 * s_ + 4; gt[5] = 4 * s_;
}
// Position of node v among a triangle's 6 nodes (6 if absent).
__device__ __forceinline__ int local_of(const int* nd, int v) {
  int i = 0;
  while (i < 6 && nd[i] != v) ++i;
  return i;
}

// FEM bending chain, the reference's sem_calculate_K_kernel and
// sem_calculate_q_kernel (sem_kernel.cu:1129-1306), one thread per node,
// gathering over the node's triangles in ascending order (the order of the
// reference's atomics under a serial schedule).  Per triangle and column l
// of the nodes' curvature tensors the 3x3 system with rows (dx/ds, dx/dt,
// n) and right-hand sides (dKapa_l/ds, dKapa_l/dt, 0) is solved; q needs
// only the diagonal K[j][j][l] of the accumulated third-order tensor:
// traceK_l = sum_j K[j][j][l] / count, q = (I - n n) traceK.
template <class R, class Pos>
__device__ __forceinline__ void fem_q(int NN, int Em, const int* tri, const int* node_ntri, const int* node_tri,
                                      const int* vert_local, const R* nNp, const R* kap, R* qv, Pos P3) {
  for (int v = threadIdx.x; v < NN; v += blockDim.x) {
    const int cnt = node_ntri[v];
    R Kd[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // [j][l]
    for (int j = 0; j < cnt; ++j) {
      const int t = node_tri[10 * v + j];
      const int* nd = tri + 6 * t;
      const int li = v < Em ? vert_local[10 * v + j] : local_of(nd, v);
      if (li > 5) continue;  // not a node of t: the lists are built from tri, so never
      R c[6][3];
      P3(nd[0], c[0]); P3(nd[1], c[1]); P3(nd[2], c[2]);
      for (int i = 0; i < 3; ++i) {
        c[3][i] = (R)0.5 * (c[0][i] + c[1][i]);
        c[4][i] = (R)0.5 * (c[0][i] + c[2][i]);
        c[5][i] = (R)0.5 * (c[1][i] + c[2][i]);
      }
      R gs[6], gt[6];
      p2_grad<R>(li, gs, gt);
      R a1[3], a3[3];
      for (int d = 0; d < 3; ++d) {
        a1[d] = c[0][d] * gs[0] + c[1][d] * gs[1] + c[2][d] * gs[2] + c[3][d] * gs[3] + c[4][d] * gs[4] +
                c[5][d] * gs[5];
        a3[d] = c[0][d] * gt[0] + c[1][d] * gt[1] + c[2][d] * gt[2] + c[3][d] * gt[3] + c[4][d] * gt[4] +
                c[5][d] * gt[5];
      }
      for (int l = 0; l < 3; ++l) {
        R g[3][6];
        for (int d = 0; d < 3; ++d) {
          R a2 = 0, a4 = 0;
          for (int m = 0; m < 6; ++m) a2 += kap[9 * nd[m] + 3 * d + l] * gs[m];
          for (int m = 0; m < 6; ++m) a4 += kap[9 * nd[m] + 3 * d + l] * gt[m];
          g[0][d] = a1[d]; g[1][d] = a3[d]; g[2][d] = nNp[3 * nd[li] + d];
          g[0][3 + d] = a2; g[1][3 + d] = a4; g[2][3 + d] = 0;
        }
        gauss36<R>(g);
        // diagonal entries A[d][d] of the solution rows
        const R A22 = g[2][5];
        const R A11 = g[1][4] - g[2][4] * g[1][2];
        const R A0_2 = g[2][3];
        const R A0_1 = g[1][3] - A0_2 * g[1][2];
        const R A00 = g[0][3] - A0_2 * g[0][2] - A0_1 * g[0][1];
        Kd[0][l] += A00;
        Kd[1][l] += A11;
        Kd[2][l] += A22;
      }
    }
    R qq[3] = {0, 0, 0};
    if (cnt > 0) {
      const R n[3] = {nNp[3 * v], nNp[3 * v + 1], nNp[3 * v + 2]};
      for (int i = 0; i < 3; ++i) {
        const R tr = Kd[0][i] / (R)cnt + Kd[1][i] / (R)cnt + Kd[2][i] / (R)cnt;
        for (int j = 0; j < 3; ++j) qq[j] += tr * ((i == j ? (R)1 : (R)0) - n[i] * n[j]);
      }
    }
    qv[3 * v] = qq[0]; qv[3 * v + 1] = qq[1]; qv[3 * v + 2] = qq[2];
  }
}

// The reference's sem_bending_force_kernel (sem_kernel.cu:1308-1497), one
// thread per triangle: unit side tangents t, in-plane normals b = t x n at
// the six nodes (the vertices also along their second side), line loads
// f = (b . q) n and Simpson's rule along the sides.  The load goes to
// ft[t]; the vertices gather it.
template <class R, class Pos>
__device__ __forceinline__ void fem_loads(int T, const int* tri, const R* nNp, const R* qv, R* ft, Pos P3) {
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    const int* nd = tri + 6 * t;
    R c[3][3], nv[6][3], tv[6][3], L[3], f[6][6];
    P3(nd[0], c[0]); P3(nd[1], c[1]); P3(nd[2], c[2]);
    for (int i = 0; i < 6; ++i)
      for (int d = 0; d < 3; ++d) nv[i][d] = nNp[3 * nd[i] + d];
    for (int d = 0; d < 3; ++d) {
      tv[0][d] = c[0][d] - c[1][d];
      tv[1][d] = c[1][d] - c[2][d];
      tv[2][d] = c[2][d] - c[0][d];
    }
    for (int i = 0; i < 3; ++i) L[i] = nrm3(tv[i][0], tv[i][1], tv[i][2]);
    for (int d = 0; d < 3; ++d) {
      tv[3][d] = tv[0][d] / L[0];
      tv[4][d] = tv[2][d] / L[2];
      tv[5][d] = tv[1][d] / L[1];
    }
    for (int i = 0; i < 3; ++i)
      for (int d = 0; d < 3; ++d) tv[i][d] /= L[i];
    for (int i = 0; i < 6; ++i) {
      R b[3];
      b[0] = tv[i][1] * nv[i][2] - tv[i][2] * nv[i][1];
      b[1] = tv[i][2] * nv[i][0] - tv[i][0] * nv[i][2];
      b[2] = tv[i][0] * nv[i][1] - tv[i][1] * nv[i][0];
      const R nb = nrm3(b[0], b[1], b[2]);
      for (int d = 0; d < 3; ++d) b[d] /= nb;
      const R* q = qv + 3 * nd[i];
      const R bq = b[0] * q[0] + b[1] * q[1] + b[2] * q[2];
      for (int d = 0; d < 3; ++d) f[i][d] = bq * nv[i][d];
      if (i < 3) {
        const R* o = tv[i == 0 ? 2 : i - 1];  // t2 at vertex 0, t0 at 1, t1 at 2
        b[0] = o[1] * nv[i][2] - o[2] * nv[i][1];
        b[1] = o[2] * nv[i][0] - o[0] * nv[i][2];
        b[2] = o[0] * nv[i][1] - o[1] * nv[i][0];
        const R nb2 = nrm3(b[0], b[1], b[2]);
        for (int d = 0; d < 3; ++d) b[d] /= nb2;
        const R bq2 = b[0] * q[0] + b[1] * q[1] + b[2] * q[2];
        for (int d = 0; d < 3; ++d) f[i][d + 3] = bq2 * nv[i][d];
      }
    }
    for (int d = 0; d < 3; ++d)
      ft[3 * t + d] = (R)0.5 * (((R)(1 / 3.0) * (f[0][d] + f[1][d + 3]) + (R)(4.0 / 3.0) * f[3][d]) * L[0] +
                                ((R)(1 / 3.0) * (f[1][d] + f[2][d + 3]) + (R)(4.0 / 3.0) * f[5][d]) * L[1] +
                                ((R)(1 / 3.0) * (f[2][d] + f[0][d + 3]) + (R)(4.0 / 3.0) * f[4][d]) * L[2]);
  }
}

// One CTA per platelet: springs + wall, triangle areas/normals and the global
// area/volume (FP64 sums), nodal normals, curvature tensor and mean
// curvature at the vertices, area/volume penalty and bending forces.  Every
// accumulation is a gather in ascending triangle order, so the result does
// not depend on scheduling.
template <class R>
__global__ void __launch_bounds__(512) membrane_k(PlateletConst k, const double* X, const double* Y,
                                                  const double* RY, const double* Z, const int* tri,
                                                  const int* node_ntri, const int* node_tri,
                                                  const int* vert_local, const int* ring, const int* sp_ptr,
                                                  const int* sp_nbr, const double* sp_L0, const double* S0,
                                                  const double* S0_all, const double* V0, R* nN, R* nelem, R* S,
                                                  R* kmv, double* SV, R* Fmem, Control* ctl, R* fem) {
  if (ctl->done) return;
  const int p = blockIdx.x;
  const int E = k.E, Em = k.Em, T = k.T, NN = k.NN, PE = k.P * k.E;
  const int base = p * E;
  const R F0 = (R)k.f0;
  // FP32 build: positions relative to the platelet's first element, cached
  // once in shared memory (x, y, z, ry); FP64 build: absolute FP64 positions
  // as the reference uses them
  constexpr bool rel = sizeof(R) == 4;
  extern __shared__ float s_pos[];
  const double ox = rel ? X[base] : 0.0, oy = rel ? Y[base] : 0.0, oz = rel ? Z[base] : 0.0;
  const double ory = rel ? RY[base] : 0.0;
  if constexpr (rel) {
    for (int e = threadIdx.x; e < E; e += blockDim.x) {
      s_pos[4 * e] = (float)(X[base + e] - ox);
      s_pos[4 * e + 1] = (float)(Y[base + e] - oy);
      s_pos[4 * e + 2] = (float)(Z[base + e] - oz);
      s_pos[4 * e + 3] = (float)(RY[base + e] - ory);
    }
    __syncthreads();
  }
  auto P3 = [&](int e, R out[3]) {
    if constexpr (rel) {
      out[0] = (R)s_pos[4 * e]; out[1] = (R)s_pos[4 * e + 1]; out[2] = (R)s_pos[4 * e + 2];
    } else {
      out[0] = (R)X[base + e]; out[1] = (R)Y[base + e]; out[2] = (R)Z[base + e];
    }
  };
  R* nNp = nN + (size_t)p * NN * 3;
  R* nep = nelem + (size_t)p * T * 3;
  R* Sp = S + (size_t)p * T;
  R* kmp = kmv + (size_t)p * Em;
  // FEM bending chain (mask PF_MEM_FEMBEND): per platelet the symmetrised
  // curvature tensors of all nodes [NN][9], the q vectors [NN][3], the
  // triangles' bending loads [T][3] and areas [T]
  const bool use_fem = (k.mask & PF_MEM_FEMBEND) && fem;
  R* kapp = use_fem ? fem + (size_t)p * ((size_t)NN * 12 + (size_t)T * 4) : nullptr;
  R* qvp = kapp ? kapp + (size_t)NN * 9 : nullptr;
  R* ftp = kapp ? qvp + (size_t)NN * 3 : nullptr;
  R* arp = kapp ? ftp + (size_t)T * 3 : nullptr;
  __shared__ double s_a[512], s_b[512];
  __shared__ int s_i[512];
  __shared__ double s_Sall, s_V;
  __shared__ int s_wall_idx;
  __shared__ double s_wall_f;

  // lowest element (sem_kernel.cu:409-430): first index attaining the minimum
  {
    double zmin = 1e300;
    int imin = 0x7fffffff;
    for (int e = threadIdx.x; e < E; e += blockDim.x) {
      const double zz = Z[base + e];
      if (zz < zmin || (zz == zmin && e < imin)) { zmin = zz; imin = e; }
    }
    s_a[threadIdx.x] = zmin;
    s_i[threadIdx.x] = imin;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        const double z2 = s_a[threadIdx.x + s];
        const int i2 = s_i[threadIdx.x + s];
        if (z2 < s_a[threadIdx.x] || (z2 == s_a[threadIdx.x] && i2 < s_i[threadIdx.x])) {
          s_a[threadIdx.x] = z2;
          s_i[threadIdx.x] = i2;
        }
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      s_wall_idx = -1;
      s_wall_f = 0;
      const double dmin = s_a[0];
      if ((k.mask & PF_MEM_WALL) && E > 0 && dmin <= 0.02) {
        s_wall_idx = s_i[0];
        s_wall_f = 5e-4 * 2000 * exp(-2000 * dmin) / (1 - exp(-2000 * dmin)) / (double)k.f0;
      }
    }
    __syncthreads();
  }
  // springs on RY (sem_kernel.cu:355-389) plus the wall force
  for (int e = threadIdx.x; e < E; e += blockDim.x) {
    R fx = 0, fy = 0, fz = 0;
    if (e == s_wall_idx && e != 0) fz = (R)s_wall_f;
    if (k.mask & PF_MEM_SPRING)
      for (int q = sp_ptr[e]; q < sp_ptr[e + 1]; ++q) {
        const int nb = sp_nbr[q];
        R d1, d2, d3;
        if constexpr (rel) {
          d1 = s_pos[4 * nb] - s_pos[4 * e];
          d2 = s_pos[4 * nb + 3] - s_pos[4 * e + 3];
          d3 = s_pos[4 * nb + 2] - s_pos[4 * e + 2];
        } else {
          d1 = X[base + nb] - X[base + e];
          d2 = RY[base + nb] - RY[base + e];
          d3 = Z[base + nb] - Z[base + e];
        }
        const R r = nrm3(d1, d2, d3);
        const R w = r - (R)sp_L0[q];
        const R fc = (R)k.kspring * w / r;
        fx += fc * d1 / (R)1.0 / F0;
        fy += fc * d2 / (R)1.0 / F0;
        fz += fc * d3 / (R)1.0 / F0;
      }
    if (e == s_wall_idx && e == 0) fz += (R)s_wall_f;
    Fmem[base + e] = fx;
    Fmem[PE + base + e] = fy;
    Fmem[2 * PE + base + e] = fz;
  }
  if (!(k.mask & (PF_MEM_AREAVOL | PF_MEM_BEND)) && !use_fem) {
    if (threadIdx.x == 0) { SV[2 * p] = 0; SV[2 * p + 1] = 0; }
    return;
  }
  // triangle areas, normals; the global area and volume are summed in FP64;
  // the local strain (Se - S0e)/S0e is kept for the area force
  double pa = 0, pv = 0;
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    const int* nd = tri + 6 * t;
    R c0[3], c1[3], c2[3];
    P3(nd[0], c0); P3(nd[1], c1); P3(nd[2], c2);
    R e12[3], e13[3], n[3], cc[3];
    for (int i = 0; i < 3; ++i) {
      cc[i] = (R)(1 / 3.0) * (c0[i] + c1[i] + c2[i]);
      e12[i] = c1[i] - c0[i];
      e13[i] = c2[i] - c0[i];
    }
    n[0] = e12[1] * e13[2] - e12[2] * e13[1];
    n[1] = e12[2] * e13[0] - e12[0] * e13[2];
    n[2] = e12[0] * e13[1] - e12[1] * e13[0];
    const R nn = nrm3(n[0], n[1], n[2]);
    n[0] /= -nn; n[1] /= -nn; n[2] /= -nn;
    const R St = (R)0.5 * nn;
    const R S0e = (R)S0[(size_t)p * T + t];
    Sp[t] = (St - S0e) / S0e;
    if (arp) arp[t] = St;
    nep[3 * t] = n[0]; nep[3 * t + 1] = n[1]; nep[3 * t + 2] = n[2];
    pa += (double)St;
    pv += (double)((R)(1 / 3.0) * (cc[0] * n[0] + cc[1] * n[1] + cc[2] * n[2]) * St);
  }
  s_a[threadIdx.x] = pa;
  s_b[threadIdx.x] = pv;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      s_a[threadIdx.x] += s_a[threadIdx.x + s];
      s_b[threadIdx.x] += s_b[threadIdx.x + s];
    }
    __syncthreads();
  }
  __shared__ double s_sglob, s_vglob;
  if (threadIdx.x == 0) {
    s_Sall = s_a[0];
    s_V = s_b[0];
    SV[2 * p] = s_a[0];
    SV[2 * p + 1] = s_b[0];
    // the relative area and volume errors, formed once per platelet
    s_sglob = (s_a[0] - S0_all[p]) / S0_all[p];
    s_vglob = (s_b[0] - V0[p]) / V0[p];
  }
  __syncthreads();
  // nodal normals: mean of the element normals of the node's triangles
  for (int q = threadIdx.x; q < NN; q += blockDim.x) {
    const int cnt = node_ntri[q];
    R a0 = 0, a1 = 0, a2 = 0;
    for (int j = 0; j < cnt; ++j) {
      const int t = node_tri[10 * q + j];
      a0 += nep[3 * t]; a1 += nep[3 * t + 1]; a2 += nep[3 * t + 2];
    }
    if (cnt > 0) {
      a0 /= (R)cnt; a1 /= (R)cnt; a2 /= (R)cnt;
      const R nn = nrm3(a0, a1, a2);
      a0 /= nn; a1 /= nn; a2 /= nn;
    }
    nNp[3 * q] = a0; nNp[3 * q + 1] = a1; nNp[3 * q + 2] = a2;
  }
  __syncthreads();
  // curvature tensor at each vertex from its triangles (6-node element),
  // mean curvature km = tr/2 of the node average; with the FEM chain at the
  // mid-side nodes too, and the symmetrised node averages kept
  const int ncurv = use_fem ? NN : Em;
  for (int v = threadIdx.x; v < ncurv; v += blockDim.x) {
    const int cnt = node_ntri[v];
    R K[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int j = 0; j < cnt; ++j) {
      const int t = node_tri[10 * v + j];
      const int* nd = tri + 6 * t;
      const int li = v < Em ? vert_local[10 * v + j] : local_of(nd, v);
      if (li > 5) continue;  // not a node of t: the lists are built from tri, so never
      R c[6][3], nv[6][3];
      P3(nd[0], c[0]); P3(nd[1], c[1]); P3(nd[2], c[2]);
      for (int i = 0; i < 3; ++i) {
        c[3][i] = (R)0.5 * (c[0][i] + c[1][i]);
        c[4][i] = (R)0.5 * (c[0][i] + c[2][i]);
        c[5][i] = (R)0.5 * (c[1][i] + c[2][i]);
      }
      for (int i = 0; i < 6; ++i)
        for (int d = 0; d < 3; ++d) nv[i][d] = nNp[3 * nd[i] + d];
      R gs[6], gt[6];
      p2_grad<R>(li, gs, gt);
      R a1[3], a2[3], a3[3], a4[3];
      for (int d = 0; d < 3; ++d) {
        a1[d] = c[0][d] * gs[0] + c[1][d] * gs[1] + c[2][d] * gs[2] + c[3][d] * gs[3] + c[4][d] * gs[4] +
                c[5][d] * gs[5];
        a2[d] = nv[0][d] * gs[0] + nv[1][d] * gs[1] + nv[2][d] * gs[2] + nv[3][d] * gs[3] + nv[4][d] * gs[4] +
                nv[5][d] * gs[5];
        a3[d] = c[0][d] * gt[0] + c[1][d] * gt[1] + c[2][d] * gt[2] + c[3][d] * gt[3] + c[4][d] * gt[4] +
                c[5][d] * gt[5];
        a4[d] = nv[0][d] * gt[0] + nv[1][d] * gt[1] + nv[2][d] * gt[2] + nv[3][d] * gt[3] + nv[4][d] * gt[4] +
                nv[5][d] * gt[5];
      }
      R A[3][3];
      {
        R g[3][6];
        for (int d = 0; d < 3; ++d) { g[0][d] = a1[d]; g[1][d] = a3[d]; g[2][d] = nv[li][d]; }
        for (int i = 0; i < 3; ++i) { g[0][3 + i] = a2[i]; g[1][3 + i] = a4[i]; g[2][3 + i] = 0; }
        gauss36<R>(g);
        for (int i = 0; i < 3; ++i) {
          A[i][2] = g[2][3 + i];
          A[i][1] = g[1][3 + i] - A[i][2] * g[1][2];
          A[i][0] = g[0][3 + i] - A[i][2] * g[0][2] - A[i][1] * g[0][1];
        }
      }
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) K[a * 3 + b] += A[b][a];
    }
    if (v < Em) {
      R km = 0;
      if (cnt > 0) km = (R)0.5 * (K[0] / (R)cnt + K[4] / (R)cnt + K[8] / (R)cnt);
      kmp[v] = km;
    }
    if (kapp)
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
          kapp[9 * v + 3 * a + b] = cnt > 0 ? (R)0.5 * (K[a * 3 + b] / (R)cnt + K[b * 3 + a] / (R)cnt) : (R)0;
  }
  __syncthreads();
  if (use_fem) {
    fem_q<R>(NN, Em, tri, node_ntri, node_tri, vert_local, nNp, kapp, qvp, P3);
    __syncthreads();
    fem_loads<R>(T, tri, nNp, qvp, ftp, P3);
    __syncthreads();
  }
  // area/volume penalty (sem_kernel.cu:1640-1749) and bending
  // (:1499-1638) at each vertex
  for (int v = threadIdx.x; v < Em; v += blockDim.x) {
    R fx = Fmem[base + v], fy = Fmem[PE + base + v], fz = Fmem[2 * PE + base + v];
    const int cnt = node_ntri[v];
    if (use_fem) {
      // each triangle's load to its vertices, divided by S[vertex id]: the
      // area of the triangle whose index is the vertex id
      // (sem_kernel.cu:1484-1495)
      const R Sv = arp[v];
      for (int j = 0; j < cnt; ++j) {
        const int t = node_tri[10 * v + j];
        fx += ftp[3 * t] / Sv / F0;
        fy += ftp[3 * t + 1] / Sv / F0;
        fz += ftp[3 * t + 2] / Sv / F0;
      }
    }
    if (k.mask & PF_MEM_AREAVOL) {
      const R Ks = (R)k.ks, Kv = (R)k.kv;
      const R sglob = (R)s_sglob, vglob = (R)s_vglob;
      for (int j = 0; j < cnt; ++j) {
        const int t = node_tri[10 * v + j];
        const int i = vert_local[10 * v + j];
        const int* nd = tri + 6 * t;
        R c[3][3], L[3][3], cc[3], n[3];
        P3(nd[0], c[0]); P3(nd[1], c[1]); P3(nd[2], c[2]);
        for (int d = 0; d < 3; ++d) {
          L[0][d] = c[1][d] - c[2][d];
          L[1][d] = c[2][d] - c[0][d];
          L[2][d] = c[0][d] - c[1][d];
          cc[d] = (R)(1 / 3.0) * (c[0][d] + c[1][d] + c[2][d]);
          n[d] = nep[3 * t + d];
        }
        R dS[3];
        dS[0] = (R)-0.5 * (L[i][1] * n[2] - L[i][2] * n[1]);
        dS[1] = (R)-0.5 * (L[i][2] * n[0] - L[i][0] * n[2]);
        dS[2] = (R)-0.5 * (L[i][0] * n[1] - L[i][1] * n[0]);
        const R fa = -Ks * (Sp[t] + sglob);
        fx += fa * dS[0] / F0;
        fy += fa * dS[1] / F0;
        fz += fa * dS[2] / F0;
        R dV[3];
        const R t0 = -L[1][1] * L[0][2] / (R)3.0 + L[1][2] * L[0][1] / (R)3.0;
        const R t1 = -L[1][2] * L[0][0] / (R)3.0 + L[1][0] * L[0][2] / (R)3.0;
        const R t2 = -L[1][0] * L[0][1] / (R)3.0 + L[1][1] * L[0][0] / (R)3.0;
        dV[0] = t0 - L[i][2] * cc[1] + L[i][1] * cc[2];
        dV[1] = t1 + L[i][2] * cc[0] - L[i][0] * cc[2];
        dV[2] = t2 - L[i][1] * cc[0] + L[i][0] * cc[1];
        const R fv = -Kv * vglob;
        fx += fv * dV[0] / (R)6.0 / F0;
        fy += fv * dV[1] / (R)6.0 / F0;
        fz += fv * dV[2] / (R)6.0 / F0;
      }
    }
    if (k.mask & PF_MEM_BEND) {
      const int* rg = ring + 10 * v;
      R xi[3], ni[3] = {nNp[3 * v], nNp[3 * v + 1], nNp[3 * v + 2]};
      P3(v, xi);
      R Ai = 0, sum = 0;
      const R kmi = kmp[v];
      for (int a = 0; a < cnt; ++a) {
        const int jn = rg[a], jp = rg[a == 0 ? cnt - 1 : a - 1], jx = rg[a == cnt - 1 ? 0 : a + 1];
        R xj[3], x1[3], x2[3];
        P3(jn, xj); P3(jp, x1); P3(jx, x2);
        R ri1[3], r1j[3], rij[3], ri2[3], r2j[3], cij[3], ci2[3], c2j[3], ce[3];
        for (int d = 0; d < 3; ++d) {
          ri1[d] = xi[d] - x1[d]; r1j[d] = x1[d] - xj[d]; rij[d] = xi[d] - xj[d];
          ri2[d] = xi[d] - x2[d]; r2j[d] = x2[d] - xj[d];
          cij[d] = (R)0.5 * (xi[d] + xj[d]); ci2[d] = (R)0.5 * (xi[d] + x2[d]); c2j[d] = (R)0.5 * (x2[d] + xj[d]);
        }
        const R ai = rij[0] * ri2[0] + rij[1] * ri2[1] + rij[2] * ri2[2];
        const R a2 = -(ri2[0] * r2j[0] + ri2[1] * r2j[1] + ri2[2] * r2j[2]);
        const R aj = rij[0] * r2j[0] + rij[1] * r2j[1] + rij[2] * r2j[2];
        const R a1 = -(r1j[0] * ri1[0] + r1j[1] * ri1[1] + r1j[2] * ri1[2]);
        if (ai < 0) {
          for (int d = 0; d < 3; ++d) ce[d] = c2j[d];
        } else if (a2 < 0) {
          for (int d = 0; d < 3; ++d) ce[d] = cij[d];
        } else if (aj < 0) {
          for (int d = 0; d < 3; ++d) ce[d] = ci2[d];
        } else {
          R g[3][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}};
          for (int d = 0; d < 3; ++d) {
            g[0][d] = rij[d]; g[1][d] = ri2[d];
            g[0][3] += cij[d] * rij[d]; g[1][3] += ci2[d] * ri2[d];
          }
          g[2][0] = (xj[1] - xi[1]) * (x2[2] - xi[2]) - (xj[2] - xi[2]) * (x2[1] - xi[1]);
          g[2][1] = (xj[2] - xi[2]) * (x2[0] - xi[0]) - (xj[0] - xi[0]) * (x2[2] - xi[2]);
          g[2][2] = (xj[0] - xi[0]) * (x2[1] - xi[1]) - (xj[1] - xi[1]) * (x2[0] - xi[0]);
          g[2][3] = g[2][0] * xi[0] + g[2][1] * xi[1] + g[2][2] * xi[2];
          gauss34<R>(g);
          ce[2] = g[2][3];
          ce[1] = g[1][3] - ce[2] * g[1][2];
          ce[0] = g[0][3] - ce[2] * g[0][2] - ce[1] * g[0][1];
        }
        R L1 = nrm3(xi[0] - cij[0], xi[1] - cij[1], xi[2] - cij[2]);
        R L2 = nrm3(ce[0] - cij[0], ce[1] - cij[1], ce[2] - cij[2]);
        const R L3 = nrm3(xi[0] - ce[0], xi[1] - ce[1], xi[2] - ce[2]);
        R Pe = (R)0.5 * (L1 + L2 + L3);
        Ai += sqrt(Pe * (Pe - L1) * (Pe - L2) * (Pe - L3));
        L1 = nrm3(xi[0] - ci2[0], xi[1] - ci2[1], xi[2] - ci2[2]);
        L2 = nrm3(ce[0] - ci2[0], ce[1] - ci2[1], ce[2] - ci2[2]);
        Pe = (R)0.5 * (L1 + L2 + L3);
        Ai += sqrt(Pe * (Pe - L1) * (Pe - L2) * (Pe - L3));
        const R ca = a1 / (nrm3(xi[0] - x1[0], xi[1] - x1[1], xi[2] - x1[2]) *
                           nrm3(x1[0] - xj[0], x1[1] - xj[1], x1[2] - xj[2]));
        const R cb = a2 / (nrm3(xi[0] - x2[0], xi[1] - x2[1], xi[2] - x2[2]) *
                           nrm3(x2[0] - xj[0], x2[1] - xj[1], x2[2] - xj[2]));
        R alpha, beta;
        if constexpr (sizeof(R) == 8) {
          alpha = (R)1 / tan(acos(ca));  // sem_kernel.cu:1624-1625
          beta = (R)1 / tan(acos(cb));
        } else {
          alpha = ca * rsqrtf(1.f - ca * ca);  // cot(acos(c)) = c / sqrt(1 - c^2)
          beta = cb * rsqrtf(1.f - cb * cb);
        }
        sum += (R)0.5 * (alpha + beta) * (kmp[jn] - kmi);
      }
      const R Kb = (R)k.kbend;
      fx += Kb / Ai * sum * ni[0] / F0;
      fy += Kb / Ai * sum * ni[1] / F0;
      fz += Kb / Ai * sum * ni[2] / F0;
    }
    Fmem[base + v] = fx;
    Fmem[PE + base + v] = fy;
    Fmem[2 * PE + base + v] = fz;
  }
}

// FP32 membrane pass with the per-vertex loops split into items: one CTA of
// kMem32Threads per platelet, every intermediate in shared memory.
//   items: (vertex v, j-th triangle of v) for the curvature trace and the
//   area/volume gradient, (vertex v, j-th ring neighbour) for the bending
//   geometry; each item writes its own slot and the per-vertex sums run over
//   the slots in j order, so the result does not depend on scheduling.
// Arithmetic differs from membrane_k<float> in the rounding only:
//   - tangents a1 = dx/ds, a3 = dx/dt of the 6-node element whose mid-side
//     nodes sit at the side midpoints are exactly c1 - c0 and c2 - c0;
//   - the curvature tensor is used through its trace, tr(A) with
//     A^T = M^-1 [a2 a4 0]^T, M = rows (a1, a3, n), by the adjugate:
//     tr = (a2 . (a3 x n) + a4 . (n x a1)) / det M;
//   - the circumcentre of (xi, xj, x2) is solved relative to xi, where the
//     right-hand side is -|r|^2/2 for the two edges and 0 for the normal.
constexpr int kMem32Threads = 512;
constexpr int kMem32Slots = 10;  // triangles / ring neighbours per vertex

struct Mem32Layout {
  int cap;  // item slots: 3 T (one per triangle corner)
  size_t pos, fs, nel, sst, nN, km, res, off, cnt, tri, item, itri, bytes;
  __host__ __device__ Mem32Layout(const PlateletConst& k) {
    cap = 3 * k.T;
    size_t o = 0;
    auto take = [&](size_t n, size_t sz) {
      const size_t at = o;
      o += (n * sz + 15) & ~(size_t)15;
      return at;
    };
    pos = take((size_t)k.E, sizeof(float4));
    fs = take((size_t)3 * k.E, sizeof(float));
    nel = take((size_t)3 * k.T, sizeof(float));
    sst = take((size_t)k.T, sizeof(float));
    nN = take((size_t)3 * k.NN, sizeof(float));
    km = take((size_t)k.Em, sizeof(float));
    res = take((size_t)6 * cap, sizeof(float));
    off = take((size_t)k.Em + 1, sizeof(int));
    cnt = take((size_t)k.NN, sizeof(int));
    tri = take((size_t)6 * k.T, sizeof(int));
    item = take((size_t)cap, sizeof(int));
    itri = take((size_t)cap, sizeof(int));
    bytes = o;
  }
};

__device__ __forceinline__ void cross3(const float a[3], const float b[3], float c[3]) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ __forceinline__ float dot3(const float a[3], const float b[3]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
__device__ __forceinline__ float len3(const float a[3]) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ void ld3(const float4* p, int e, float c[3]) {
  const float4 v = p[e];
  c[0] = v.x; c[1] = v.y; c[2] = v.z;
}
// Heron's formula; the product is clamped at zero (a right triangle whose
// hypotenuse equals a leg in floating point has a zero factor).
__device__ __forceinline__ float heron(float l1, float l2, float l3) {
  const float pe = 0.5f * (l1 + l2 + l3);
  return sqrtf(fmaxf(0.f, pe * (pe - l1) * (pe - l2) * (pe - l3)));
}

__device__ __forceinline__ void membrane32_k_body(const PlateletConst& k, const double* X, const double* Y, const double* RY, const double* Z,
                 const int* tri, const int* node_ntri, const int* node_tri, const int* vert_local, const int* ring,
                 const int* sp_ptr, const int* sp_nbr, const double* sp_L0, const double* S0,
                 const double* S0_all, const double* V0, float* kmv, double* SV, float* Fmem, Control* ctl, int bid, int nblk) {
  if (ctl->done) return;
  constexpr int NT = kMem32Threads, NW = NT / 32;
  const int p = bid, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int E = k.E, Em = k.Em, T = k.T, NN = k.NN, PE = k.P * k.E;
  const int base = p * E;
  const float invF0 = 1.f / k.f0;
  const Mem32Layout lay(k);
  extern __shared__ __align__(16) unsigned char smem[];
  float4* s_pos = reinterpret_cast<float4*>(smem + lay.pos);
  float* s_fs = reinterpret_cast<float*>(smem + lay.fs);
  float* s_nel = reinterpret_cast<float*>(smem + lay.nel);
  float* s_sst = reinterpret_cast<float*>(smem + lay.sst);
  float* s_nN = reinterpret_cast<float*>(smem + lay.nN);
  float* s_km = reinterpret_cast<float*>(smem + lay.km);
  float* s_res = reinterpret_cast<float*>(smem + lay.res);
  int* s_off = reinterpret_cast<int*>(smem + lay.off);
  int* s_cnt = reinterpret_cast<int*>(smem + lay.cnt);
  int* s_tri = reinterpret_cast<int*>(smem + lay.tri);
  int* s_item = reinterpret_cast<int*>(smem + lay.item);
  int* s_itri = reinterpret_cast<int*>(smem + lay.itri);
  const int cap = lay.cap;
  float* r_tr = s_res;              // curvature trace of item
  float* r_av = s_res + cap;        // area/volume force of item, 3 components
  float* r_area = s_res + 4 * cap;  // bending: mixed area of the item's sector
  float* r_w = s_res + 5 * cap;     // bending: 0.5 (cot alpha + cot beta)
  __shared__ double s_da[NW], s_db[NW];
  __shared__ int s_di[NW], s_ws[NW];
  __shared__ int s_wall_idx, s_total;
  __shared__ float s_wall_f;
  __shared__ double s_Sall, s_V;
  __shared__ float s_sglob, s_vglob;

  // phase 0: positions relative to element 0, the lowest element, node
  // triangle counts and triangles staged, per-thread sums of the vertex
  // triangle counts (a contiguous chunk of vertices per thread)
  const double ox = X[base], oy = Y[base], oz = Z[base], ory = RY[base];
  double zmin = 1e300;
  int imin = 0x7fffffff;
  for (int e = tid; e < E; e += NT) {
    const double zz = Z[base + e];
    s_pos[e] = make_float4((float)(X[base + e] - ox), (float)(Y[base + e] - oy), (float)(zz - oz),
                           (float)(RY[base + e] - ory));
    if (zz < zmin) { zmin = zz; imin = e; }  // e ascending: first index of the minimum
  }
  for (int q = tid; q < NN; q += NT) s_cnt[q] = node_ntri[q];
  for (int i = tid; i < 6 * T; i += NT) s_tri[i] = tri[i];
  const int chunk = (Em + NT - 1) / NT;
  const int v0 = min(Em, tid * chunk), v1 = min(Em, v0 + chunk);
  int mine = 0;
  for (int v = v0; v < v1; ++v) mine += node_ntri[v];
  int incl = mine;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double z2 = __shfl_xor_sync(0xffffffffu, zmin, o);
    const int i2 = __shfl_xor_sync(0xffffffffu, imin, o);
    if (z2 < zmin || (z2 == zmin && i2 < imin)) { zmin = z2; imin = i2; }
  }
  if (lane == 0) { s_da[wid] = zmin; s_di[wid] = imin; }
  if (lane == 31) s_ws[wid] = incl;
  __syncthreads();
  if (tid == 0) {
    double zm = s_da[0];
    int im = s_di[0];
    for (int w = 1; w < NW; ++w)
      if (s_da[w] < zm || (s_da[w] == zm && s_di[w] < im)) { zm = s_da[w]; im = s_di[w]; }
    s_wall_idx = -1;
    s_wall_f = 0.f;
    if ((k.mask & PF_MEM_WALL) && E > 0 && zm <= 0.02) {
      s_wall_idx = im;
      s_wall_f = (float)(5e-4 * 2000 * exp(-2000 * zm) / (1 - exp(-2000 * zm)) / (double)k.f0);
    }
  }
  // exclusive offsets of this thread's vertices: earlier warps' totals plus
  // the inclusive scan within the warp, less this thread's own sum
  {
    int before = 0, total = 0;
    for (int w = 0; w < NW; ++w) {
      const int s = s_ws[w];
      before += w < wid ? s : 0;
      total += s;
    }
    int run = before + incl - mine;
    for (int v = v0; v < v1; ++v) {
      s_off[v] = run;
      run += s_cnt[v];
    }
    if (tid == 0) { s_off[Em] = total; s_total = total; }
  }
  const bool surface = (k.mask & (PF_MEM_AREAVOL | PF_MEM_BEND)) != 0;
  __syncthreads();
  if (surface && s_total > cap) {  // a vertex listed in more triangles than it has corners
    if (tid == 0) atomicOr(&ctl->err, ERR_MEMBRANE_SIZE);
    return;
  }

  // phase 1: springs on RY plus the wall force (sem_kernel.cu:355-389);
  // triangle normals, strains, FP64 area and volume sums; the item table
  const int wall = s_wall_idx;
  for (int e = tid; e < E; e += NT) {
    float fx = 0.f, fy = 0.f, fz = 0.f;
    if (e == wall && e != 0) fz = s_wall_f;
    if (k.mask & PF_MEM_SPRING) {
      const float4 pe = s_pos[e];
      for (int q = sp_ptr[e]; q < sp_ptr[e + 1]; ++q) {
        const float4 pn = s_pos[sp_nbr[q]];
        const float d1 = pn.x - pe.x, d2 = pn.w - pe.w, d3 = pn.z - pe.z;
        const float r = sqrtf(d1 * d1 + d2 * d2 + d3 * d3);
        const float fc = k.kspring * (r - (float)sp_L0[q]) / r * invF0;
        fx += fc * d1;
        fy += fc * d2;
        fz += fc * d3;
      }
    }
    if (e == wall && e == 0) fz += s_wall_f;
    s_fs[3 * e] = fx;
    s_fs[3 * e + 1] = fy;
    s_fs[3 * e + 2] = fz;
  }
  if (!surface) {
    __syncthreads();
    for (int e = tid; e < E; e += NT) {
      Fmem[base + e] = s_fs[3 * e];
      Fmem[PE + base + e] = s_fs[3 * e + 1];
      Fmem[2 * PE + base + e] = s_fs[3 * e + 2];
    }
    if (tid == 0) { SV[2 * p] = 0; SV[2 * p + 1] = 0; }
    return;
  }
  double pa = 0, pv = 0;
  for (int t = tid; t < T; t += NT) {
    const int* nd = s_tri + 6 * t;
    float c0[3], c1[3], c2[3], e12[3], e13[3], n[3];
    ld3(s_pos, nd[0], c0); ld3(s_pos, nd[1], c1); ld3(s_pos, nd[2], c2);
    for (int i = 0; i < 3; ++i) { e12[i] = c1[i] - c0[i]; e13[i] = c2[i] - c0[i]; }
    cross3(e12, e13, n);
    const float nn = len3(n);
    const float ninv = -1.f / nn;
    for (int i = 0; i < 3; ++i) n[i] *= ninv;
    const float St = 0.5f * nn;
    const float S0e = (float)S0[(size_t)p * T + t];
    s_sst[t] = (St - S0e) / S0e;
    s_nel[3 * t] = n[0]; s_nel[3 * t + 1] = n[1]; s_nel[3 * t + 2] = n[2];
    float cc[3];
    for (int i = 0; i < 3; ++i) cc[i] = (1.f / 3.f) * (c0[i] + c1[i] + c2[i]);
    pa += (double)St;
    pv += (double)((1.f / 3.f) * dot3(cc, n) * St);
  }
  for (int v = tid; v < Em; v += NT) {
    const int o = s_off[v], c = s_cnt[v];
    for (int j = 0; j < c; ++j) {
      s_item[o + j] = (v << 4) | j;
      s_itri[o + j] = (node_tri[kMem32Slots * v + j] << 2) | vert_local[kMem32Slots * v + j];
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    pa += __shfl_xor_sync(0xffffffffu, pa, o);
    pv += __shfl_xor_sync(0xffffffffu, pv, o);
  }
  if (lane == 0) { s_da[wid] = pa; s_db[wid] = pv; }
  __syncthreads();

  // phase 2: nodal normals (mean of the element normals, normalised); the
  // global area and volume
  if (tid == 0) {
    double a = 0, b = 0;
    for (int w = 0; w < NW; ++w) { a += s_da[w]; b += s_db[w]; }
    s_Sall = a;
    s_V = b;
    SV[2 * p] = a;
    SV[2 * p + 1] = b;
    // the relative area and volume errors, formed once: FP64 divisions in
    // every thread would hold the SM's narrow FP64 pipe for microseconds
    s_sglob = (float)((a - S0_all[p]) / S0_all[p]);
    s_vglob = (float)((b - V0[p]) / V0[p]);
  }
  for (int q = tid; q < NN; q += NT) {
    const int cnt = s_cnt[q];
    float a[3] = {0.f, 0.f, 0.f};
    for (int j = 0; j < cnt; ++j) {
      const int t = node_tri[kMem32Slots * q + j];
      a[0] += s_nel[3 * t]; a[1] += s_nel[3 * t + 1]; a[2] += s_nel[3 * t + 2];
    }
    if (cnt > 0) {
      // mean then normalise: the 1/cnt factor cancels in the direction
      const float inv = rsqrtf(dot3(a, a));
      for (int i = 0; i < 3; ++i) a[i] *= inv;
    }
    s_nN[3 * q] = a[0]; s_nN[3 * q + 1] = a[1]; s_nN[3 * q + 2] = a[2];
  }
  __syncthreads();

  // phase 3: items -- curvature trace, area/volume gradient
  // (sem_kernel.cu:1640-1749), bending geometry (:1499-1638)
  const int total = s_total;
  const float sglob = s_sglob, vglob = s_vglob;
  for (int it = tid; it < 3 * total; it += NT) {
    const int kind = it >= total ? (it >= 2 * total ? 2 : 1) : 0;
    const int i = it - kind * total;
    if (kind == 0) {
      const int t = s_itri[i] >> 2, li = s_itri[i] & 3;
      const int* nd = s_tri + 6 * t;
      float c0[3], c1[3], c2[3], a1[3], a3[3], a2[3] = {0.f, 0.f, 0.f}, a4[3] = {0.f, 0.f, 0.f};
      ld3(s_pos, nd[0], c0); ld3(s_pos, nd[1], c1); ld3(s_pos, nd[2], c2);
      for (int d = 0; d < 3; ++d) { a1[d] = c1[d] - c0[d]; a3[d] = c2[d] - c0[d]; }
      const float s_ = li == 1 ? 1.f : 0.f, t_ = li == 2 ? 1.f : 0.f;
      const float gs[6] = {4 * s_ + 4 * t_ - 3, 4 * s_ - 1, 0, -8 * s_ - 4 * t_ + 4, -4 * t_, 4 * t_};
      const float gt[6] = {4 * t_ + 4 * s_ - 3, 0, 4 * t_ - 1, -4 * s_, -8 * t_ - 4 * s_ + 4, 4 * s_};
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        const int nq = nd[q];
        for (int d = 0; d < 3; ++d) {
          const float nv = s_nN[3 * nq + d];
          a2[d] += nv * gs[q];
          a4[d] += nv * gt[q];
        }
      }
      const int nl_ = li == 0 ? nd[0] : li == 1 ? nd[1] : nd[2];
      const float nl[3] = {s_nN[3 * nl_], s_nN[3 * nl_ + 1], s_nN[3 * nl_ + 2]};
      float q0[3], q1[3];
      cross3(a3, nl, q0);
      cross3(nl, a1, q1);
      r_tr[i] = (dot3(a2, q0) + dot3(a4, q1)) / dot3(a1, q0);
    } else if (kind == 1) {
      const int t = s_itri[i] >> 2, li = s_itri[i] & 3;
      const int* nd = s_tri + 6 * t;
      float c0[3], c1[3], c2[3], L0[3], L1[3], Li[3], cc[3], n[3];
      ld3(s_pos, nd[0], c0); ld3(s_pos, nd[1], c1); ld3(s_pos, nd[2], c2);
      for (int d = 0; d < 3; ++d) {
        L0[d] = c1[d] - c2[d];
        L1[d] = c2[d] - c0[d];
        Li[d] = li == 0 ? L0[d] : li == 1 ? L1[d] : c0[d] - c1[d];
        cc[d] = (1.f / 3.f) * (c0[d] + c1[d] + c2[d]);
        n[d] = s_nel[3 * t + d];
      }
      float f[3] = {0.f, 0.f, 0.f};
      if (k.mask & PF_MEM_AREAVOL) {
        float dS[3], lc[3], t01[3];
        cross3(Li, n, dS);
        cross3(L0, L1, t01);
        cross3(Li, cc, lc);
        const float fa = -0.5f * -k.ks * (s_sst[t] + sglob) * invF0;
        const float fv = -k.kv * vglob * (1.f / 6.f) * invF0;
        for (int d = 0; d < 3; ++d) f[d] = fa * dS[d] + fv * (t01[d] * (1.f / 3.f) + lc[d]);
      }
      r_av[i] = f[0]; r_av[cap + i] = f[1]; r_av[2 * cap + i] = f[2];
    } else {
      const int v = s_item[i] >> 4, j = s_item[i] & 15;
      const int cnt = s_cnt[v];
      const int* rg = ring + kMem32Slots * v;
      const int jn = rg[j], jp = rg[j == 0 ? cnt - 1 : j - 1], jx = rg[j == cnt - 1 ? 0 : j + 1];
      float xi[3], xj[3], x1[3], x2[3];
      ld3(s_pos, v, xi); ld3(s_pos, jn, xj); ld3(s_pos, jp, x1); ld3(s_pos, jx, x2);
      float rij[3], ri2[3], r2j[3], ri1[3], r1j[3];
      for (int d = 0; d < 3; ++d) {
        rij[d] = xi[d] - xj[d]; ri2[d] = xi[d] - x2[d]; r2j[d] = x2[d] - xj[d];
        ri1[d] = xi[d] - x1[d]; r1j[d] = x1[d] - xj[d];
      }
      const float ai = dot3(rij, ri2), a2 = -dot3(ri2, r2j), aj = dot3(rij, r2j), a1 = -dot3(r1j, ri1);
      // circumcentre ce = xi + w; h = xi - (xi+xj)/2, h2 = xi - (xi+x2)/2
      float w[3], h[3], h2[3];
      for (int d = 0; d < 3; ++d) { h[d] = 0.5f * rij[d]; h2[d] = 0.5f * ri2[d]; }
      if (ai < 0) {
        for (int d = 0; d < 3; ++d) w[d] = -0.5f * (rij[d] + ri2[d]);
      } else if (a2 < 0) {
        for (int d = 0; d < 3; ++d) w[d] = -h[d];
      } else if (aj < 0) {
        for (int d = 0; d < 3; ++d) w[d] = -h2[d];
      } else {
        float nrm[3], u0[3], u1[3];
        cross3(rij, ri2, nrm);
        cross3(ri2, nrm, u0);
        cross3(nrm, rij, u1);
        const float dinv = 1.f / dot3(rij, u0);
        const float d0 = -0.5f * dot3(rij, rij) * dinv, d1 = -0.5f * dot3(ri2, ri2) * dinv;
        for (int d = 0; d < 3; ++d) w[d] = d0 * u0[d] + d1 * u1[d];
      }
      float wh[3], wh2[3];
      for (int d = 0; d < 3; ++d) { wh[d] = w[d] + h[d]; wh2[d] = w[d] + h2[d]; }
      const float L3 = len3(w);
      r_area[i] = heron(len3(h), len3(wh), L3) + heron(len3(h2), len3(wh2), L3);
      // cot(acos(c)) = c / sqrt(1 - c^2), c the cosine of the angle at x1 / x2
      const float ca = a1 * rsqrtf(dot3(ri1, ri1) * dot3(r1j, r1j));
      const float cb = a2 * rsqrtf(dot3(ri2, ri2) * dot3(r2j, r2j));
      r_w[i] = 0.5f * (ca * rsqrtf(1.f - ca * ca) + cb * rsqrtf(1.f - cb * cb));
    }
  }
  __syncthreads();

  // phase 4: mean curvature km = tr / 2 of the node average
  for (int v = tid; v < Em; v += NT) {
    const int o = s_off[v], cnt = s_cnt[v];
    float tr = 0.f;
    for (int j = 0; j < cnt; ++j) tr += r_tr[o + j];
    const float km = cnt > 0 ? 0.5f * (tr / (float)cnt) : 0.f;
    s_km[v] = km;
    kmv[(size_t)p * Em + v] = km;
  }
  __syncthreads();

  // phase 5: element force = springs + area/volume + bending
  const float Kb = k.kbend * invF0;
  for (int e = tid; e < E; e += NT) {
    float fx = s_fs[3 * e], fy = s_fs[3 * e + 1], fz = s_fs[3 * e + 2];
    if (e < Em) {
      const int o = s_off[e], cnt = s_cnt[e];
      if (k.mask & PF_MEM_AREAVOL)
        for (int j = 0; j < cnt; ++j) {
          fx += r_av[o + j];
          fy += r_av[cap + o + j];
          fz += r_av[2 * cap + o + j];
        }
      if (k.mask & PF_MEM_BEND) {
        const int* rg = ring + kMem32Slots * e;
        const float kmi = s_km[e];
        float Ai = 0.f, sum = 0.f;
        for (int j = 0; j < cnt; ++j) {
          Ai += r_area[o + j];
          sum += r_w[o + j] * (s_km[rg[j]] - kmi);
        }
        const float g = Kb * sum / Ai;
        fx += g * s_nN[3 * e];
        fy += g * s_nN[3 * e + 1];
        fz += g * s_nN[3 * e + 2];
      }
    }
    Fmem[base + e] = fx;
    Fmem[PE + base + e] = fy;
    Fmem[2 * PE + base + e] = fz;
  }
}
__global__ void __launch_bounds__(kMem32Threads, 2)
    membrane32_k(PlateletConst k, const double* X, const double* Y, const double* RY, const double* Z,
                 const int* tri, const int* node_ntri, const int* node_tri, const int* vert_local, const int* ring,
                 const int* sp_ptr, const int* sp_nbr, const double* sp_L0, const double* S0,
                 const double* S0_all, const double* V0, float* kmv, double* SV, float* Fmem, Control* ctl) {
  membrane32_k_body(k, X, Y, RY, Z, tri, node_ntri, node_tri, vert_local, ring, sp_ptr, sp_nbr, sp_L0, S0, S0_all, V0, kmv, SV, Fmem, ctl, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------- Morse
// FP32 Morse force over distance, F(r)/r, force-shifted to zero at the
// cutoff: (2 rho U0 (e^2 - e) - F(rc)) / r with e = exp(rho (req - r)),
// evaluated without a branch (e = 2^(K1 - K2 r), K2 = rho log2(e),
// K1 = K2 req); zero outside 0 < r^2 < rc^2.
struct MorseF32 {
  float rc2, K1, K2, A, Fc;
  __host__ __device__ MorseF32(const double prm[4], double fc) {
    const float rho = (float)prm[1], rc = (float)prm[3];
    rc2 = rc * rc;
    K2 = rho * 1.44269504088896341f;
    K1 = K2 * (float)prm[2];
    A = 2.0f * rho * (float)prm[0];
    Fc = (float)fc;
  }
};
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float morse_fr(const MorseF32& m, float r2) {
  const bool in = r2 < m.rc2 && r2 > 0.f;
  const float rinv = rsqrtf(in ? r2 : 1.f);
  const float ex = ex2_approx(fmaf(-m.K2, r2 * rinv, m.K1));
  const float fr = fmaf(m.A, ex * (ex - 1.f), -m.Fc) * rinv;
  return in ? fr : 0.f;
}
// Cell bins are sorted by element id after binning, so a cell list is the
// same set in the same order as the oracle's counting sort, and the pair sums
// below run in a fixed order.
__global__ void __launch_bounds__(256) sort_bins_k(int ncells, const int* bin_count, float4* bin,
                                                   const Control* ctl) {
  if (ctl->done) return;
  const int* occ = reinterpret_cast<const int*>(bin + (size_t)ncells * kBinCap);
  const int nocc = ctl->occupied;
  __shared__ float4 s_b[kBinCap];
  for (int oc = blockIdx.x; oc < nocc; oc += gridDim.x) {
    const int c = occ[oc];
    const int cnt = min(bin_count[c], kBinCap);
    int pow2 = 1;
    while (pow2 < cnt) pow2 <<= 1;
    float4* b = bin + (size_t)c * kBinCap;
    for (int i = threadIdx.x; i < pow2; i += blockDim.x)
      s_b[i] = i < cnt ? b[i] : make_float4(0, 0, 0, __int_as_float(0x7fffffff));
    __syncthreads();
    for (int size = 2; size <= pow2; size <<= 1)
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        for (int i = threadIdx.x; i < pow2; i += blockDim.x) {
          const int j = i ^ stride;
          if (j > i) {
            const bool up = (i & size) == 0;
            const float4 a = s_b[i], e = s_b[j];
            if ((__float_as_int(a.w) > __float_as_int(e.w)) == up) { s_b[i] = e; s_b[j] = a; }
          }
        }
        __syncthreads();
      }
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) b[i] = s_b[i];
    __syncthreads();
  }
}

// F_i = sum_j 2 rho U0 [e^{2 rho (req - r)} - e^{rho (req - r)}] (x_i - x_j)/r
// for 0 < r < cutoff (intra- or inter-platelet parameters), over the 27
// neighbouring cells in a fixed order.  One CTA per occupied cell: the cell's
// elements are the threads; each neighbour cell's members are staged through
// shared memory and read by broadcast.  FP32 build: cell-relative float
// coordinates from the bins (no FP64 in the pair loop).  FP64 build, or a
// periodic axis with fewer than three cells: FP64 positions, minimum image,
// neighbour cells de-duplicated.
template <class R, bool FAST>
__global__ void __launch_bounds__(128) morse_k(PlateletConst k, const double* X, const double* Y, const double* Z,
                                               const int* bin_count, const float4* bin, double* Fm, Control* ctl) {
  if (ctl->done) return;
  const int PE = k.P * k.E;
  const int ncells = k.ncell[0] * k.ncell[1] * k.ncell[2];
  const int* occ = reinterpret_cast<const int*>(bin + (size_t)ncells * kBinCap);
  const int nocc = ctl->occupied;
  __shared__ float4 s_m[128];
  const R U0a = (R)k.morse_intra[0], rhoa = (R)k.morse_intra[1], reqa = (R)k.morse_intra[2], rca = (R)k.morse_intra[3];
  const R U0b = (R)k.morse_inter[0], rhob = (R)k.morse_inter[1], reqb = (R)k.morse_inter[2], rcb = (R)k.morse_inter[3];
  const R rc2a = rca * rca, rc2b = rcb * rcb;
  const R Fca = (R)k.morse_fc[0], Fcb = (R)k.morse_fc[1];
  const float cs0 = (float)k.cs[0], cs1 = (float)k.cs[1], cs2 = (float)k.cs[2];
  for (int oc = blockIdx.x; oc < nocc; oc += gridDim.x) {
    const int c = occ[oc];
    const int cnt = min(bin_count[c], kBinCap);
    const int c0 = c % k.ncell[0], c1 = (c / k.ncell[0]) % k.ncell[1], c2 = c / (k.ncell[0] * k.ncell[1]);
    for (int q0 = 0; q0 < cnt; q0 += blockDim.x) {
      const int q = q0 + threadIdx.x;
      const bool valid = q < cnt;
      const float4 own = valid ? bin[(size_t)c * kBinCap + q] : make_float4(0, 0, 0, __int_as_float(-1));
      const int g = __float_as_int(own.w);
      const int pbase = valid ? (g / k.E) * k.E : 0;
      double xi = 0, yi = 0, zi = 0;
      if (!FAST && valid) { xi = X[g]; yi = Y[g]; zi = Z[g]; }
      R ax = 0, ay = 0, az = 0;
      int seen[FAST ? 1 : 27];
      int nseen = 0;
      for (int nb = 0; nb < 27; ++nb) {
        const int dx = nb % 3 - 1, dy = (nb / 3) % 3 - 1, dz = nb / 9 - 1;
        int cc0 = c0 + dx, cc1 = c1 + dy, cc2 = c2 + dz;
        if (cc0 < 0 || cc0 >= k.ncell[0]) { if (!k.wrap[0]) continue; cc0 = (cc0 + k.ncell[0]) % k.ncell[0]; }
        if (cc1 < 0 || cc1 >= k.ncell[1]) { if (!k.wrap[1]) continue; cc1 = (cc1 + k.ncell[1]) % k.ncell[1]; }
        if (cc2 < 0 || cc2 >= k.ncell[2]) { if (!k.wrap[2]) continue; cc2 = (cc2 + k.ncell[2]) % k.ncell[2]; }
        const int nc = cc0 + k.ncell[0] * (cc1 + k.ncell[1] * cc2);
        if (!FAST) {
          bool dup = false;
          for (int t = 0; t < nseen; ++t) dup |= (seen[t] == nc);
          if (dup) continue;
          seen[nseen++] = nc;
        }
        const int ncnt = min(bin_count[nc], kBinCap);
        const float ox = own.x - dx * cs0, oy = own.y - dy * cs1, oz = own.z - dz * cs2;
        for (int m0 = 0; m0 < ncnt; m0 += 128) {
          __syncthreads();
          if (m0 + threadIdx.x < ncnt) s_m[threadIdx.x] = bin[(size_t)nc * kBinCap + m0 + threadIdx.x];
          __syncthreads();
          const int mm = min(128, ncnt - m0);
          if (!valid) continue;
#pragma unroll 4
          for (int j = 0; j < mm; ++j) {
            const float4 mb = s_m[j];
            const int h = __float_as_int(mb.w);
            const bool intra = (unsigned)(h - pbase) < (unsigned)k.E;
            R d0, d1, d2;
            if (FAST) {
              d0 = (R)(ox - mb.x); d1 = (R)(oy - mb.y); d2 = (R)(oz - mb.z);
            } else {
              double e0 = xi - X[h], e1 = yi - Y[h], e2 = zi - Z[h];
              if (k.wrap[0]) e0 -= k.L[0] * floor(e0 / k.L[0] + 0.5);
              if (k.wrap[1]) e1 -= k.L[1] * floor(e1 / k.L[1] + 0.5);
              if (k.wrap[2]) e2 -= k.L[2] * floor(e2 / k.L[2] + 0.5);
              d0 = (R)e0; d1 = (R)e1; d2 = (R)e2;
            }
            const R r2 = d0 * d0 + d1 * d1 + d2 * d2;
            if (!(r2 < (intra ? rc2a : rc2b)) || !(r2 > (R)0)) continue;
            const R U0 = intra ? U0a : U0b, rho = intra ? rhoa : rhob, req = intra ? reqa : reqb;
            const R Fc = intra ? Fca : Fcb;
            R fr;
            if (sizeof(R) == 4) {
              const float rinv = rsqrtf((float)r2);
              const float r = (float)r2 * rinv;
              const float ex = __expf((float)rho * ((float)req - r));
              fr = (R)((2.0f * (float)rho * (float)U0 * (ex * ex - ex) - (float)Fc) * rinv);
            } else {
              const R r = sqrt(r2);
              if (!(r < (intra ? rca : rcb))) continue;
              const R ex = exp(rho * (req - r));
              fr = ((R)2.0 * rho * U0 * (ex * ex - ex) - Fc) / r;
            }
            ax += fr * d0; ay += fr * d1; az += fr * d2;
          }
        }
      }
      if (valid && g >= 0 && g < PE) {
        const double sc = k.inv_f0;
        Fm[g] = (double)ax * sc;
        Fm[PE + g] = (double)ay * sc;
        Fm[2 * PE + g] = (double)az * sc;
      }
    }
  }
}

// Per-platelet all-pairs Morse (platelets of at most kMorseTileE elements):
// the platelet's elements, relative to its first element with the minimum
// image, are staged in shared memory; several CTAs share a platelet, each
// owning a slice of its elements; other platelets whose bounding spheres come
// within the inter-platelet cutoff are staged and scanned the same way.  Same
// pair set and formula as the cell-list kernel, summed in element order.
constexpr int kMorseTileE = 2048;

// Per platelet: centroid (minimum image about the first element), bounding
// radius about the centroid, and every element's position relative to the
// centroid -- float in the FP32 build, double in the FP64 build -- written
// once per step so the pair kernel stages plain loads.
template <class R>
struct Staged;
template <>
struct Staged<float> {
  using T = float4;
  static __device__ __forceinline__ T make(double x, double y, double z, int id) {
    return make_float4((float)x, (float)y, (float)z, __int_as_float(id));
  }
  static __device__ __forceinline__ T shift(T a, double ox, double oy, double oz) {
    return make_float4(a.x + (float)ox, a.y + (float)oy, a.z + (float)oz, a.w);
  }
};
template <>
struct Staged<double> {
  using T = D4;
  static __device__ __forceinline__ T make(double x, double y, double z, int id) { return D4{x, y, z, (double)id}; }
  static __device__ __forceinline__ T shift(T a, double ox, double oy, double oz) {
    return D4{a.x + ox, a.y + oy, a.z + oz, a.w};
  }
};

template <class T = double>
__device__ __forceinline__ T min_image(T d, T L, int wrap) {
  if (!wrap) return d;
  if (d > (T)0.5 * L) d -= L;
  else if (d < (T)-0.5 * L) d += L;
  return d;
}

constexpr int kBoundsThreads = 512;
template <class R>
__device__ __forceinline__ void platelet_bounds_k_body(const PlateletConst& k, const double* X,
                                                                    const double* Y, const double* Z,
                                                                    double* bounds, typename Staged<R>::T* rel,
                                                                    const Control* ctl, int bid, int nblk) {
  if (ctl->done) return;
  constexpr int NW = kBoundsThreads / 32;
  const int p = bid, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int base = p * k.E;
  const double ox = X[base], oy = Y[base], oz = Z[base];
  __shared__ R s_w[3][NW];
  __shared__ double s_c[3];
  __shared__ R s_r[NW];
  // centroid: minimum-image offsets from the first element, summed per
  // thread, per warp, then over the warps in order.  The FP32 build forms
  // each offset with one FP64 subtraction and sums in FP32 (the centroid
  // only fixes the frame of the float positions; FP64 is slow on this GPU)
  R sx = 0, sy = 0, sz = 0;
  const R Lx = (R)k.L[0], Ly = (R)k.L[1], Lz = (R)k.L[2];
  for (int e = threadIdx.x; e < k.E; e += kBoundsThreads) {
    sx += min_image<R>((R)(X[base + e] - ox), Lx, k.wrap[0]);
    sy += min_image<R>((R)(Y[base + e] - oy), Ly, k.wrap[1]);
    sz += min_image<R>((R)(Z[base + e] - oz), Lz, k.wrap[2]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    sx += __shfl_xor_sync(0xffffffffu, sx, o);
    sy += __shfl_xor_sync(0xffffffffu, sy, o);
    sz += __shfl_xor_sync(0xffffffffu, sz, o);
  }
  if (lane == 0) { s_w[0][wid] = sx; s_w[1][wid] = sy; s_w[2][wid] = sz; }
  __syncthreads();
  if (threadIdx.x < 3) {
    R t = 0;
    for (int w = 0; w < NW; ++w) t += s_w[threadIdx.x][w];
    s_c[threadIdx.x] = (threadIdx.x == 0 ? ox : threadIdx.x == 1 ? oy : oz) + (double)(t / (R)k.E);
  }
  __syncthreads();
  const double cx_ = s_c[0], cy_ = s_c[1], cz_ = s_c[2];
  // positions relative to the centroid, and the bounding radius
  R r2max = 0;
  for (int e = threadIdx.x; e < k.E; e += kBoundsThreads) {
    const R d0 = min_image<R>((R)(X[base + e] - cx_), Lx, k.wrap[0]);
    const R d1 = min_image<R>((R)(Y[base + e] - cy_), Ly, k.wrap[1]);
    const R d2 = min_image<R>((R)(Z[base + e] - cz_), Lz, k.wrap[2]);
    rel[base + e] = Staged<R>::make(d0, d1, d2, base + e);
    r2max = fmax(r2max, d0 * d0 + d1 * d1 + d2 * d2);
  }
  for (int o = 16; o > 0; o >>= 1) r2max = fmax(r2max, __shfl_xor_sync(0xffffffffu, r2max, o));
  if (lane == 0) s_r[wid] = r2max;
  __syncthreads();
  if (threadIdx.x == 0) {
    R m = 0;
    for (int w = 0; w < NW; ++w) m = fmax(m, s_r[w]);
    bounds[4 * p] = cx_; bounds[4 * p + 1] = cy_; bounds[4 * p + 2] = cz_;
    bounds[4 * p + 3] = sqrt((double)m);
  }
}
template <class R>
__global__ void __launch_bounds__(kBoundsThreads) platelet_bounds_k(PlateletConst k, const double* X,
                                                                    const double* Y, const double* Z,
                                                                    double* bounds, typename Staged<R>::T* rel,
                                                                    const Control* ctl) {
  platelet_bounds_k_body<R>(k, X, Y, Z, bounds, rel, ctl, blockIdx.x, gridDim.x);
}

// 32 elements per CTA, each element's partner list split over kMorseSplit
// warps; the partial sums are added in warp order (deterministic).
constexpr int kMorseSplit = 4;

template <class R>
__device__ __forceinline__ void morse_platelet_k_body(const PlateletConst& k, const double* bounds,
                                                                     const typename Staged<R>::T* rel,
                                                                     int tiles, double* Fm, Control* ctl, int bid, int nblk) {
  if (ctl->done) return;
  using T = typename Staged<R>::T;
  extern __shared__ __align__(16) unsigned char s_raw[];
  T* s_t = reinterpret_cast<T*>(s_raw);
  T* s_q = s_t + k.E;
  __shared__ R s_part[kMorseSplit][3][32];
  const int PE = k.P * k.E;
  const int p = bid / tiles, tile = bid % tiles;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int e = tile * 32 + lane;
  const bool valid = e < k.E;
  const double cxp = bounds[4 * p], cyp = bounds[4 * p + 1], czp = bounds[4 * p + 2], rp = bounds[4 * p + 3];
  for (int j = threadIdx.x; j < k.E; j += blockDim.x) s_t[j] = rel[p * k.E + j];
  __syncthreads();
  const R U0a = (R)k.morse_intra[0], rhoa = (R)k.morse_intra[1], reqa = (R)k.morse_intra[2];
  const R rca = (R)k.morse_intra[3], rc2a = rca * rca, Fca = (R)k.morse_fc[0];
  const R U0b = (R)k.morse_inter[0], rhob = (R)k.morse_inter[1], reqb = (R)k.morse_inter[2];
  const R rcb = (R)k.morse_inter[3], rc2b = rcb * rcb, Fcb = (R)k.morse_fc[1];
  const T own = valid ? s_t[e] : Staged<R>::make(0, 0, 0, 0);
  R ax = 0, ay = 0, az = 0;
  const MorseF32 fa(k.morse_intra, k.morse_fc[0]), fb(k.morse_inter, k.morse_fc[1]);
  // FP32: branchless (every lane evaluates, out-of-range pairs add zero)
  auto pair32 = [&](const T mb, const MorseF32& m) {
    const float d0 = (float)own.x - (float)mb.x, d1 = (float)own.y - (float)mb.y, d2 = (float)own.z - (float)mb.z;
    const float fr = morse_fr(m, d0 * d0 + d1 * d1 + d2 * d2);
    ax += fr * d0; ay += fr * d1; az += fr * d2;
  };
  auto pair = [&](const T mb, R U0, R rho, R req, R rc, R rc2, R Fc) {
    const R d0 = (R)own.x - (R)mb.x, d1 = (R)own.y - (R)mb.y, d2 = (R)own.z - (R)mb.z;
    const R r2 = d0 * d0 + d1 * d1 + d2 * d2;
    if (!(r2 < rc2) || !(r2 > (R)0)) return;
    R fr;
    if constexpr (sizeof(R) == 4) {
      const float rinv = rsqrtf(r2);
      const float r = r2 * rinv;
      const float ex = __expf(rho * (req - r));
      fr = (2.0f * rho * U0 * (ex * ex - ex) - Fc) * rinv;
    } else {
      const R r = sqrt(r2);
      if (!(r < rc)) return;
      const R ex = exp(rho * (req - r));
      fr = ((R)2.0 * rho * U0 * (ex * ex - ex) - Fc) / r;
    }
    ax += fr * d0; ay += fr * d1; az += fr * d2;
  };
  const int chunk = (k.E + kMorseSplit - 1) / kMorseSplit;
  const int j0 = w * chunk, j1 = min(k.E, j0 + chunk);
  if (valid) {
    if constexpr (sizeof(R) == 4) {
#pragma unroll 4
      for (int j = j0; j < j1; ++j) pair32(s_t[j], fa);
    } else {
      for (int j = j0; j < j1; ++j) pair(s_t[j], U0a, rhoa, reqa, rca, rc2a, Fca);
    }
  }
  // Other platelets whose bounding spheres come within the inter cutoff,
  // shifted into this platelet's centroid frame (minimum image).  The
  // candidates are found in chunks of blockDim platelets, one per thread, and
  // compacted in ascending platelet order into shared memory, so the per-pair
  // loop below sees only offsets of type R.
  __shared__ R s_off[32 * kMorseSplit][4];
  __shared__ int s_qid[32 * kMorseSplit];
  __shared__ int s_wcount[kMorseSplit];
  for (int qb = 0; qb < k.P; qb += blockDim.x) {
    const int q = qb + threadIdx.x;
    bool near = false;
    double o0 = 0, o1 = 0, o2 = 0, rq = 0;
    if (q < k.P && q != p) {
      o0 = min_image(bounds[4 * q] - cxp, k.L[0], k.wrap[0]);
      o1 = min_image(bounds[4 * q + 1] - cyp, k.L[1], k.wrap[1]);
      o2 = min_image(bounds[4 * q + 2] - czp, k.L[2], k.wrap[2]);
      rq = bounds[4 * q + 3];
      const double reach = rp + rq + k.morse_inter[3];
      near = o0 * o0 + o1 * o1 + o2 * o2 < reach * reach;
    }
    const unsigned ball = __ballot_sync(0xffffffffu, near);
    __syncthreads();  // the previous chunk's list is no longer read
    if (lane == 0) s_wcount[w] = __popc(ball);
    __syncthreads();
    int before = 0, nq = 0;
    for (int t = 0; t < kMorseSplit; ++t) {
      if (t < w) before += s_wcount[t];
      nq += s_wcount[t];
    }
    if (near) {
      const int slot = before + __popc(ball & ((1u << lane) - 1u));
      s_qid[slot] = q;
      s_off[slot][0] = (R)o0;
      s_off[slot][1] = (R)o1;
      s_off[slot][2] = (R)o2;
      s_off[slot][3] = (R)(rq + k.morse_inter[3]) * (R)1.0001 + (R)1e-6;
    }
    __syncthreads();
    for (int i = 0; i < nq; ++i) {
      const int qq = s_qid[i];
      const R f0 = s_off[i][0], f1 = s_off[i][1], f2 = s_off[i][2], lim = s_off[i][3];
      __syncthreads();  // s_q of the previous platelet is no longer read
      for (int j = threadIdx.x; j < k.E; j += blockDim.x) {
        T a = rel[qq * k.E + j];
        a.x += f0; a.y += f1; a.z += f2;
        s_q[j] = a;
      }
      __syncthreads();
      if (!valid) continue;
      // this element is out of reach of platelet qq: skip its members
      const R dq0 = (R)own.x - f0, dq1 = (R)own.y - f1, dq2 = (R)own.z - f2;
      if (dq0 * dq0 + dq1 * dq1 + dq2 * dq2 >= lim * lim) continue;
      if constexpr (sizeof(R) == 4) {
        for (int j = j0; j < j1; ++j) pair32(s_q[j], fb);
      } else {
        for (int j = j0; j < j1; ++j) pair(s_q[j], U0b, rhob, reqb, rcb, rc2b, Fcb);
      }
    }
  }
  s_part[w][0][lane] = ax;
  s_part[w][1][lane] = ay;
  s_part[w][2][lane] = az;
  __syncthreads();
  if (w == 0 && valid) {
    R sx = 0, sy = 0, sz = 0;
    for (int t = 0; t < kMorseSplit; ++t) { sx += s_part[t][0][lane]; sy += s_part[t][1][lane]; sz += s_part[t][2][lane]; }
    const int g = p * k.E + e;
    const R sc = (R)k.inv_f0;
    Fm[g] = (double)(sx * sc);
    Fm[PE + g] = (double)(sy * sc);
    Fm[2 * PE + g] = (double)(sz * sc);
  }
}
template <class R>
__global__ void __launch_bounds__(32 * kMorseSplit) morse_platelet_k(PlateletConst k, const double* bounds,
                                                                     const typename Staged<R>::T* rel,
                                                                     int tiles, double* Fm, Control* ctl) {
  morse_platelet_k_body<R>(k, bounds, rel, tiles, Fm, ctl, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------- fibrin
template <class R>
__device__ __forceinline__ void fibrin_k_body(int M, int law, double kk, double mass, const double* X, const double* Y, const double* Z,
                         const int* ptr, const int* nbr, const double* L0, double* F, const Control* ctl, int bid, int nblk) {
  if (ctl->done) return;
  const int ni = bid * blockDim.x + threadIdx.x;
  if (ni >= M) return;
  R fx = 0, fy = 0, fz = 0;
  const double xi = X[ni], yi = Y[ni], zi = Z[ni];
  for (int q = ptr[ni]; q < ptr[ni + 1]; ++q) {
    const int o = nbr[q];
    const R d0 = (R)(xi - X[o]), d1 = (R)(yi - Y[o]), d2 = (R)(zi - Z[o]);
    const R len = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    if (len < (R)1.0e-13) continue;
    const R l0 = (R)L0[q];
    R wf;
    if (law == PF_FIB_WLC) {
      const R En = (R)(1.3806503 * 1e-8 * 10);
      const R CC = En / l0;
      const R tl = (R)1.0 - (len - l0) / l0;
      const R IP1 = (R)0.25 * (R)1.0 / (tl * tl) - (R)0.25 + (len - l0) / l0;
      wf = -CC * IP1 / (R)mass;
    } else {
      wf = (R)kk * (len - l0);
    }
    fx -= wf * d0 / len;
    fy -= wf * d1 / len;
    fz -= wf * d2 / len;
  }
  F[ni] = (double)fx;
  F[M + ni] = (double)fy;
  F[2 * M + ni] = (double)fz;
}
// Reduced precision with four lanes per fibrin node: lane c takes the node's
// links c, c+4, ... (the per-link arithmetic of fibrin_k_body), the lanes'
// sums are added as (s0 + s1) + (s2 + s3).  The per-node loop is a chain of
// dependent loads (link list, neighbour position); four short chains in
// flight instead of one long one.
constexpr int kFibLanes = 4;
__global__ void __launch_bounds__(128) fibrin4_k(int M, int law, double kk, double mass, const double* X,
                                                 const double* Y, const double* Z, const int* ptr, const int* nbr,
                                                 const double* L0, double* F, const Control* ctl) {
  if (ctl->done) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int ni = t / kFibLanes, c = t % kFibLanes;
  const bool live = ni < M;
  float fx = 0, fy = 0, fz = 0;
  if (live) {
    const double xi = X[ni], yi = Y[ni], zi = Z[ni];
    const int q1 = ptr[ni + 1];
    for (int q = ptr[ni] + c; q < q1; q += kFibLanes) {
      const int o = nbr[q];
      const float d0 = (float)(xi - X[o]), d1 = (float)(yi - Y[o]), d2 = (float)(zi - Z[o]);
      const float len = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
      if (len < 1.0e-13f) continue;
      const float l0 = (float)L0[q];
      float wf;
      if (law == PF_FIB_WLC) {
        const float En = (float)(1.3806503 * 1e-8 * 10);
        const float CC = En / l0;
        const float tl = 1.0f - (len - l0) / l0;
        const float IP1 = 0.25f * 1.0f / (tl * tl) - 0.25f + (len - l0) / l0;
        wf = -CC * IP1 / (float)mass;
      } else {
        wf = (float)kk * (len - l0);
      }
      fx -= wf * d0 / len;
      fy -= wf * d1 / len;
      fz -= wf * d2 / len;
    }
  }
#pragma unroll
  for (int o = 1; o < kFibLanes; o <<= 1) {
    fx += __shfl_xor_sync(0xffffffffu, fx, o);
    fy += __shfl_xor_sync(0xffffffffu, fy, o);
    fz += __shfl_xor_sync(0xffffffffu, fz, o);
  }
  if (live && c == 0) {
    F[ni] = (double)fx;
    F[M + ni] = (double)fy;
    F[2 * M + ni] = (double)fz;
  }
}

template <class R>
__global__ void fibrin_k(int M, int law, double kk, double mass, const double* X, const double* Y, const double* Z,
                         const int* ptr, const int* nbr, const double* L0, double* F, const Control* ctl) {
  fibrin_k_body<R>(M, law, kk, mass, X, Y, Z, ptr, nbr, L0, F, ctl, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------- bonds
struct RecTmp {
  double ds[3], dc[3];  // receptor minus anchor for the stored site and the claim site
  double drv[3];        // receptor to each vertex of its triangle
  int bond0, si, sj, ci, cj;
  int kind[2];  // 0 none, 1 claim, 2 release
  int ok[2];
};

__device__ __forceinline__ unsigned long long op_key(int site, int rid, int opi) {
  return ((unsigned long long)(unsigned)site << 32) | ((unsigned long long)(unsigned)rid << 1) |
         (unsigned long long)opi;
}

// Bond pass, part 1 (all receptors, many CTAs): receptor positions, Bell or
// constant probabilities, decisions from the two injected uniforms, and the
// slot operations they imply.  Receptors on the triangle above the bond
// range and unbound do nothing (sem_kernel.cu:1812).  Every receptor reads
// totalBond before any addition: avaiBond = NUMOFRECEPTORS.
__device__ __forceinline__ void bonds_prepare_k_body(const PlateletConst& k, const double* X, const double* Y, const double* Z,
                                const int* tri, const int* rec_tri, const float* r1a, const float* r2a,
                                const int* rec_state, RecTmp* tmp, int* active, unsigned long long* ops, int ops_cap,
                                void* Fbond, int fbond_bytes, Control* ctl, int bid, int nblk) {
  if (ctl->done) return;
  const int PE = k.P * k.E;
  const int NR = k.P * k.nrec;
  const int gid = bid * blockDim.x + threadIdx.x;
  const int gsz = nblk * blockDim.x;
  for (int i = gid; i < 3 * PE * fbond_bytes / 4; i += gsz) ((int*)Fbond)[i] = 0;
  const int r = gid;
  if (r >= NR) return;
  const long long step = ctl->step;
  const double dx = k.dxd, dt = k.dtd;
  const int avai = (int)(k.numrec - 0);
  const int p = r / k.nrec;
  const int eo = p * k.E;
  const int* nd = tri + 6 * rec_tri[r];
  const int* st = rec_state + 3 * r;
  const float r1 = r1a[r], r2 = r2a[r];
  const float wa = 1 - r1, wb = r1 * (1 - r2), wc = r1 * r2;
  const double rz = wa * Z[eo + nd[0]] + wb * Z[eo + nd[1]] + wc * Z[eo + nd[2]];
  const int bond = st[2] > -1 ? st[2] : 0;
  if (rz > 0.078 && bond == 0) return;
  RecTmp t;
  t.kind[0] = t.kind[1] = 0;
  t.ok[0] = t.ok[1] = 0;
  const double rx = wa * X[eo + nd[0]] + wb * X[eo + nd[1]] + wc * X[eo + nd[2]];
  const double ry = wa * Y[eo + nd[0]] + wb * Y[eo + nd[1]] + wc * Y[eo + nd[2]];
  t.bond0 = bond;
  t.si = st[0]; t.sj = st[1];
  const int si = bond ? st[0] : (int)(rx / dx + 0.5), sj = bond ? st[1] : (int)(ry / dx + 0.5);
  t.ci = (int)(rx / dx + 0.5);
  t.cj = (int)(ry / dx + 0.5);
  t.ds[0] = rx - t.si * dx; t.ds[1] = ry - t.sj * dx; t.ds[2] = rz;
  t.dc[0] = rx - t.ci * dx; t.dc[1] = ry - t.cj * dx; t.dc[2] = rz;
  for (int m = 0; m < 3; ++m) {
    const double a1 = rx - X[eo + nd[m]], b1 = ry - Y[eo + nd[m]], c1 = rz - Z[eo + nd[m]];
    t.drv[m] = sqrt(a1 * a1 + b1 * b1 + c1 * c1);
  }
  const double d1 = rx - si * dx, d2 = ry - sj * dx, d3 = rz;
  const double dr = sqrt(d1 * d1 + d2 * d2 + d3 * d3);
  const double w = fabs(0.078 - dr);
  const double fc = 10.0 * w;
  double aon, aoff;
  if (k.bond_model == PF_BOND_BELL) {
    const double Kf = (double)k.kf0 * exp(fc * (0.00071 - 0.5 * w) / 4.05) * avai;
    const double Kr = (double)k.kr0 * exp(0.00071 * fc / 4.05) * avai;
    aon = 1 - exp(-Kf * dt);
    aoff = 1 - exp(-Kr * dt);
  } else {
    aon = k.p_on;
    aoff = k.p_off;
  }
  double u1, u2;
  receptor_uniforms(k.seed, step, r, u1, u2);
  if (bond == 0) {
    if (u1 < aon) t.kind[0] = 1;
    if (u2 < aon) t.kind[1] = 1;
  } else if (bond == 1) {
    if (u1 < aoff) {
      t.kind[0] = 2;
      if (u2 < aon && rz < 0.078) t.kind[1] = 1;
    } else if (u2 < aoff && rz < 0.078) {
      t.kind[0] = 2;
    }
  } else if (bond == 2) {
    if (u1 < aoff) t.kind[0] = 2;
    if (u2 < aoff) t.kind[1] = 2;
  }
  tmp[r] = t;
  active[atomicAdd(&ctl->nops_active[1], 1)] = r;
  for (int o = 0; o < 2; ++o) {
    if (!t.kind[o]) continue;
    const int ii = t.kind[o] == 1 ? t.ci : t.si, jj = t.kind[o] == 1 ? t.cj : t.sj;
    const int site = wrapi(jj, k.ny) * k.nx + wrapi(ii, k.nx);
    const int slot = atomicAdd(&ctl->nops_active[0], 1);
    if (slot < ops_cap) ops[slot] = op_key(site, r, o);
    else atomicOr(&ctl->err, ERR_BOND_OVERFLOW);
  }
}
__global__ void bonds_prepare_k(PlateletConst k, const double* X, const double* Y, const double* Z,
                                const int* tri, const int* rec_tri, const float* r1a, const float* r2a,
                                const int* rec_state, RecTmp* tmp, int* active, unsigned long long* ops, int ops_cap,
                                void* Fbond, int fbond_bytes, Control* ctl) {
  bonds_prepare_k_body(k, X, Y, Z, tri, rec_tri, r1a, r2a, rec_state, tmp, active, ops, ops_cap, Fbond, fbond_bytes, ctl, blockIdx.x, gridDim.x);
}

// Bond pass, part 2 (one CTA): slot operations sorted by (site, receptor,
// operation) and applied site by site in that order -- the outcome of a serial
// schedule of sem_kernel.cu:1750-2083 -- then bond counts, stored sites and
// the bond spring force on the triangle's vertices.
template <class R>
__device__ __forceinline__ void bonds_resolve_k_body(const PlateletConst& k, const double* X, const double* Y,
                                                        const double* Z, const int* tri, const int* rec_tri,
                                                        int* rec_state, int* vwf, RecTmp* tmp, const int* active,
                                                        unsigned long long* ops, int ops_cap, R* Fbond,
                                                        Control* ctl, int bid, int nblk) {
  if (ctl->done) return;
  const int PE = k.P * k.E;
  __shared__ long long s_tot[32];
  const int nops = min(ctl->nops_active[0], ops_cap);
  const int nact = ctl->nops_active[1];
  int pow2 = 1;
  while (pow2 < nops) pow2 <<= 1;
  for (int i = nops + threadIdx.x; i < pow2; i += blockDim.x) ops[i] = ~0ull;
  __syncthreads();
  for (int size = 2; size <= pow2; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < pow2; i += blockDim.x) {
        const int j = i ^ stride;
        if (j > i) {
          const bool up = (i & size) == 0;
          const unsigned long long a = ops[i], b = ops[j];
          if ((a > b) == up) { ops[i] = b; ops[j] = a; }
        }
      }
      __syncthreads();
    }
  const int plane = k.nx * k.ny;
  for (int i = threadIdx.x; i < nops; i += blockDim.x) {
    const unsigned site = (unsigned)(ops[i] >> 32);
    if (i > 0 && (unsigned)(ops[i - 1] >> 32) == site) continue;
    for (int j = i; j < nops && (unsigned)(ops[j] >> 32) == site; ++j) {
      const int rid = (int)((ops[j] >> 1) & 0x7fffffffu);
      const int o = (int)(ops[j] & 1u);
      const int kind = tmp[rid].kind[o];
      int ok = 0;
      for (int kk = 0; kk < 4; ++kk) {
        int* slot = vwf + (size_t)kk * plane + site;
        if (kind == 1 && *slot == -1) { *slot = rid; ok = 1; break; }
        if (kind == 2 && *slot == rid) { *slot = -1; ok = 1; break; }
      }
      tmp[rid].ok[o] = ok;
    }
  }
  __syncthreads();
  long long tot = 0;
  for (int a = threadIdx.x; a < nact; a += blockDim.x) {
    const int r = active[a];
    const RecTmp t = tmp[r];
    int bond = t.bond0, si = t.bond0 ? t.si : -1, sj = t.bond0 ? t.sj : -1;
    bool at_claim = false;
    for (int o = 0; o < 2; ++o) {
      if (!t.kind[o] || !t.ok[o]) continue;
      if (t.kind[o] == 1) { bond++; si = t.ci; sj = t.cj; at_claim = true; }
      else { bond--; if (bond == 0) { si = -1; sj = -1; at_claim = false; } }
    }
    int* st = rec_state + 3 * r;
    st[0] = si; st[1] = sj;
    if (bond) {
      const int p = r / k.nrec;
      const int eo = p * k.E;
      const int* nd = tri + 6 * rec_tri[r];
      const double* dv = at_claim ? t.dc : t.ds;
      const double d1 = dv[0], d2 = dv[1], d3 = dv[2];
      const double dr = sqrt(d1 * d1 + d2 * d2 + d3 * d3);
      const double fcb = 10.0 * (0.078 - dr) * bond / dr;
      const double fX = fcb * d1, fY = fcb * d2, fZ = fcb * d3;
      const double* drv = t.drv;
      const double sum = 1.0 / drv[0] + 1.0 / drv[1] + 1.0 / drv[2];
      for (int m = 0; m < 3; ++m) {
        const int e = eo + nd[m];
        atomicAdd(Fbond + e, (R)(fX * 1.0 / drv[m] / sum / (double)k.f0));
        atomicAdd(Fbond + PE + e, (R)(fY * 1.0 / drv[m] / sum / (double)k.f0));
        atomicAdd(Fbond + 2 * PE + e, (R)(fZ * 1.0 / drv[m] / sum / (double)k.f0));
      }
      st[2] = bond;
      tot += bond;
    } else {
      st[2] = -1;
    }
  }
  for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
  if ((threadIdx.x & 31) == 0) s_tot[threadIdx.x >> 5] = tot;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long sm = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) sm += s_tot[w];
    ctl->total_bond = (int)sm;
    ctl->nops = nops;
    ctl->nops_active[0] = 0;
    ctl->nops_active[1] = 0;
  }
}
template <class R>
__global__ void __launch_bounds__(1024) bonds_resolve_k(PlateletConst k, const double* X, const double* Y,
                                                        const double* Z, const int* tri, const int* rec_tri,
                                                        int* rec_state, int* vwf, RecTmp* tmp, const int* active,
                                                        unsigned long long* ops, int ops_cap, R* Fbond,
                                                        Control* ctl) {
  bonds_resolve_k_body<R>(k, X, Y, Z, tri, rec_tri, rec_state, vwf, tmp, active, ops, ops_cap, Fbond, ctl, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------- batch kernels
// One launch per kernel over all jobs of a fused batch; CTA b belongs to job
// batch_job_of(start, nj, b) and runs the job's body with its local CTA
// index.  The job's constants are copied to shared memory first.
#define PF_BATCH_PROLOGUE                                 \
  const int j = batch_job_of(start, nj, blockIdx.x);      \
  const BatchDesc& d = descs[j];                          \
  const int bid = blockIdx.x - start[j], nblk = start[j + 1] - start[j];

__global__ void __launch_bounds__(kFlagThreads) flag_batch_k(const BatchDesc* descs, const int* start, int nj) {
  PF_BATCH_PROLOGUE
  __shared__ LatticeConst s_lk;
  cta_copy(s_lk, d.L.k);
  __syncthreads();
  flag_k_body(s_lk, d.L.mark, d.L.flags[0], d.L.flags[1], d.L.list[0], d.L.list[1], nullptr, nullptr,
              kFlagR - 1, d.ctl, bid, nblk, true);
}

__global__ void __launch_bounds__(kMem32Threads, 1) membrane_batch_k(const BatchDesc* descs, const int* start,
                                                                     int nj) {
  PF_BATCH_PROLOGUE
  __shared__ PlateletConst s_pk;
  cta_copy(s_pk, d.Pl.k);
  __syncthreads();
  const Platelets& Pl = d.Pl;
  membrane32_k_body(s_pk, Pl.X, Pl.Y, Pl.RY, Pl.Z, Pl.tri, Pl.node_ntri, Pl.node_tri, Pl.vert_local, Pl.ring,
                    Pl.sp_ptr, Pl.sp_nbr, Pl.sp_L0, Pl.S0, Pl.S0_all, Pl.V0, (float*)Pl.km, Pl.SV,
                    (float*)Pl.Fmem, d.ctl, bid, nblk);
}

__global__ void __launch_bounds__(kBoundsThreads) bounds_batch_k(const BatchDesc* descs, const int* start, int nj) {
  PF_BATCH_PROLOGUE
  __shared__ PlateletConst s_pk;
  cta_copy(s_pk, d.Pl.k);
  __syncthreads();
  platelet_bounds_k_body<float>(s_pk, d.Pl.X, d.Pl.Y, d.Pl.Z, d.Pl.bounds, (float4*)d.Pl.relpos, d.ctl, bid,
                                nblk);
}

__global__ void __launch_bounds__(32 * kMorseSplit) morse_batch_k(const BatchDesc* descs, const int* start,
                                                                  int nj) {
  PF_BATCH_PROLOGUE
  __shared__ PlateletConst s_pk;
  cta_copy(s_pk, d.Pl.k);
  __syncthreads();
  morse_platelet_k_body<float>(s_pk, d.Pl.bounds, (const float4*)d.Pl.relpos, (s_pk.E + 31) / 32, d.Pl.Fmorse,
                               d.ctl, bid, nblk);
}

// the bond pass's scratch inside rec_tmp (the layout bond_pass uses)
struct BondScratch {
  RecTmp* tmp;
  int* active;
  unsigned long long* ops;
  int cap;
};
__device__ __forceinline__ BondScratch bond_scratch(const Platelets& Pl) {
  const int NR = Pl.k.P * Pl.k.nrec;
  BondScratch b;
  b.tmp = (RecTmp*)Pl.rec_tmp;
  b.active = (int*)(b.tmp + NR);
  b.ops = (unsigned long long*)(((uintptr_t)(b.active + NR) + 15) & ~(uintptr_t)15);
  b.cap = 2 * NR;
  return b;
}
__global__ void __launch_bounds__(256) bond_prep_batch_k(const BatchDesc* descs, const int* start, int nj) {
  PF_BATCH_PROLOGUE
  __shared__ PlateletConst s_pk;
  cta_copy(s_pk, d.Pl.k);
  __syncthreads();
  const Platelets& Pl = d.Pl;
  const BondScratch b = bond_scratch(Pl);
  bonds_prepare_k_body(s_pk, Pl.X, Pl.Y, Pl.Z, Pl.tri, Pl.rec_tri, Pl.r1, Pl.r2, Pl.rec_state, b.tmp, b.active,
                       b.ops, b.cap, Pl.Fbond, 4, d.ctl, bid, nblk);
}
__global__ void __launch_bounds__(1024) bond_resolve_batch_k(const BatchDesc* descs, const int* start, int nj) {
  PF_BATCH_PROLOGUE
  __shared__ PlateletConst s_pk;
  cta_copy(s_pk, d.Pl.k);
  __syncthreads();
  const Platelets& Pl = d.Pl;
  const BondScratch b = bond_scratch(Pl);
  bonds_resolve_k_body<float>(s_pk, Pl.X, Pl.Y, Pl.Z, Pl.tri, Pl.rec_tri, Pl.rec_state, Pl.vwf, b.tmp, b.active,
                              b.ops, b.cap, (float*)Pl.Fbond, d.ctl, bid, nblk);
}

__global__ void __launch_bounds__(kMarkerThreadsMax) fibrin_batch_k(const BatchDesc* descs, const int* start, int nj) {
  PF_BATCH_PROLOGUE
  const Fibrin& Fb = d.Fb;
  fibrin_k_body<float>(Fb.M, Fb.law, Fb.k, Fb.mass, Fb.X, Fb.Y, Fb.Z, Fb.ptr, Fb.nbr, Fb.L0, Fb.F, d.ctl, bid,
                       nblk);
}

// part 0: element membrane + Morse forces, 1: bond forces, 2: fibrin forces
template <int PART>
__global__ void __launch_bounds__(kMarkerThreadsMax) spread_batch_k(const BatchDesc* descs, const int* start, int nj) {
  PF_BATCH_PROLOGUE
  __shared__ LatticeConst s_lk;
  __shared__ double s_rdiv;
  cta_copy(s_lk, d.L.k);
  if (threadIdx.x == 0) s_rdiv = 1.0 / (d.has_pl ? (double)d.Pl.k.f0 : 1.0);
  __syncthreads();
  float4* FA = (float4*)d.L.F[0];
  float4* FB = (float4*)d.L.F[1];
  (void)nblk;
  if constexpr (PART == 2) {
    const Fibrin& Fb = d.Fb;
    spread4_body(s_lk, FA, FB, Fb.M, Fb.X, Fb.Y, Fb.Z, nullptr, Fb.F, s_rdiv, d.ctl, bid);
  } else {
    const Platelets& Pl = d.Pl;
    const int PE = Pl.k.P * Pl.k.E;
    spread4_body(s_lk, FA, FB, PE, Pl.X, Pl.Y, Pl.Z, (const float*)(PART == 0 ? Pl.Fmem : Pl.Fbond),
                 PART == 0 && Pl.k.morse ? Pl.Fmorse : nullptr, 1.0, d.ctl, bid);
  }
}

// Register cap (four 256-thread CTAs per SM, 64 registers): the per-job
// handles the batch form loads from its table otherwise hold about 100
// registers, and the extra warps of the cap outweigh its few spills
// (measured +0.8 % on the 64-job batched step).
__global__ void __launch_bounds__(kMarkerThreadsMax, 4) interp_batch_k(const BatchDesc* descs, const int* start, int nj) {
  PF_BATCH_PROLOGUE
  __shared__ LatticeConst s_lk;
  __shared__ PlateletConst s_pk;
  cta_copy(s_lk, d.L.k);
  cta_copy(s_pk, d.Pl.k);
  __syncthreads();
  const Platelets& Pl = d.Pl;
  const Fibrin& Fb = d.Fb;
  const bool pl = d.has_pl != 0, fb = d.has_fb != 0;
  interp_advance_k_body<float>(
      s_lk, s_pk, (const float4*)d.L.ubuf, pl ? s_pk.P * s_pk.E : 0, Pl.X, Pl.Y, Pl.RY, Pl.Z, Pl.V, fb ? Fb.M : 0,
      Fb.X, Fb.Y, Fb.Z, Fb.V, Fb.fixed, nullptr, nullptr, d.L.mark, d.ctl, d.done_blocks, d.detach_rate, d.seed,
      pl ? (const float*)Pl.Fmem : nullptr, (pl && s_pk.morse) ? Pl.Fmorse : nullptr,
      (pl && s_pk.nrec) ? (const float*)Pl.Fbond : nullptr, pl ? Pl.Ftot : nullptr, bid, nblk);
}
#undef PF_BATCH_PROLOGUE

}  // namespace

int membrane_threads() { return 512; }

// The item-parallel FP32 kernel takes a platelet whose intermediates fit in
// shared memory (about 150 KB for 600 elements, 796 six-node triangles);
// PFGPU_MEMBRANE_PER_VERTEX=1 selects the per-vertex kernel instead.
constexpr size_t kMem32MaxSmem = 200u << 10;
bool membrane_items(const PlateletConst& k) {
  if (getenv("PFGPU_MEMBRANE_PER_VERTEX")) return false;
  if (k.mask & PF_MEM_FEMBEND) return false;  // the FEM chain is in the per-vertex kernel only
  return Mem32Layout(k).bytes <= kMem32MaxSmem && k.E < (1 << 26);
}

static cudaError_t launch_mem32(const PlateletConst& k, const double* X, const double* Y, const double* RY,
                                const double* Z, const int* tri, const int* node_ntri, const int* node_tri,
                                const int* vert_local, const int* ring, const int* sp_ptr, const int* sp_nbr,
                                const double* sp_L0, const double* S0, const double* S0_all, const double* V0,
                                float* km, double* SV, float* F, Control* ctl, cudaStream_t st) {
  // the attribute is per device: set on every launch (host-only, cheap), so
  // a second device or host thread never launches without it
  const cudaError_t e =
      cudaFuncSetAttribute(membrane32_k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMem32MaxSmem);
  if (e != cudaSuccess) return e;
  membrane32_k<<<k.P, kMem32Threads, Mem32Layout(k).bytes, st>>>(k, X, Y, RY, Z, tri, node_ntri, node_tri,
                                                                 vert_local, ring, sp_ptr, sp_nbr, sp_L0, S0,
                                                                 S0_all, V0, km, SV, F, ctl);
  return cudaGetLastError();
}

cudaError_t membrane_forces(Platelets& Pl, int precision, Control* ctl, cudaStream_t st) {
  const PlateletConst& k = Pl.k;
  if (k.P == 0) return cudaSuccess;
  if (precision != PF_PREC_FP64 && Pl.mem_items)
    return launch_mem32(k, Pl.X, Pl.Y, Pl.RY, Pl.Z, Pl.tri, Pl.node_ntri, Pl.node_tri, Pl.vert_local, Pl.ring,
                        Pl.sp_ptr, Pl.sp_nbr, Pl.sp_L0, Pl.S0, Pl.S0_all, Pl.V0, (float*)Pl.km, Pl.SV,
                        (float*)Pl.Fmem, ctl, st);
  if (precision == PF_PREC_FP64)
    membrane_k<double><<<k.P, 512, 0, st>>>(k, Pl.X, Pl.Y, Pl.RY, Pl.Z, Pl.tri, Pl.node_ntri, Pl.node_tri,
                                            Pl.vert_local, Pl.ring, Pl.sp_ptr, Pl.sp_nbr, Pl.sp_L0, Pl.S0,
                                            Pl.S0_all, Pl.V0, (double*)Pl.nN, (double*)Pl.nelem, (double*)Pl.S,
                                            (double*)Pl.km, Pl.SV, (double*)Pl.Fmem, ctl, (double*)Pl.fem);
  else
    membrane_k<float><<<k.P, 512, (size_t)k.E * 4 * sizeof(float), st>>>(k, Pl.X, Pl.Y, Pl.RY, Pl.Z, Pl.tri, Pl.node_ntri, Pl.node_tri,
                                           Pl.vert_local, Pl.ring, Pl.sp_ptr, Pl.sp_nbr, Pl.sp_L0, Pl.S0,
                                           Pl.S0_all, Pl.V0, (float*)Pl.nN, (float*)Pl.nelem, (float*)Pl.S,
                                           (float*)Pl.km, Pl.SV, (float*)Pl.Fmem, ctl, (float*)Pl.fem);
  return cudaGetLastError();
}

// The membrane pass on caller-given arrays (the no-allocation entry point):
// same kernel and launch shape as membrane_forces.
cudaError_t membrane_forces_raw(const PlateletConst& k, int precision, const double* X, const double* Y,
                                const double* RY, const double* Z, const int* tri, const int* node_ntri,
                                const int* node_tri, const int* vert_local, const int* ring, const int* sp_ptr,
                                const int* sp_nbr, const double* sp_L0, const double* S0, const double* S0_all,
                                const double* V0, void* nN, void* nelem, void* S, void* km, double* SV, void* F,
                                Control* ctl, cudaStream_t st) {
  if (k.P == 0) return cudaSuccess;
  if (precision != PF_PREC_FP64 && membrane_items(k))
    return launch_mem32(k, X, Y, RY, Z, tri, node_ntri, node_tri, vert_local, ring, sp_ptr, sp_nbr, sp_L0, S0,
                        S0_all, V0, (float*)km, SV, (float*)F, ctl, st);
  if (precision == PF_PREC_FP64)
    membrane_k<double><<<k.P, 512, 0, st>>>(k, X, Y, RY, Z, tri, node_ntri, node_tri, vert_local, ring, sp_ptr,
                                            sp_nbr, sp_L0, S0, S0_all, V0, (double*)nN, (double*)nelem, (double*)S,
                                            (double*)km, SV, (double*)F, ctl, nullptr);
  else
    membrane_k<float><<<k.P, 512, (size_t)k.E * 4 * sizeof(float), st>>>(
        k, X, Y, RY, Z, tri, node_ntri, node_tri, vert_local, ring, sp_ptr, sp_nbr, sp_L0, S0, S0_all, V0,
        (float*)nN, (float*)nelem, (float*)S, (float*)km, SV, (float*)F, ctl, nullptr);
  return cudaGetLastError();
}

bool morse_uses_cells(const PlateletConst& k) { return k.E > kMorseTileE; }


cudaError_t morse_forces(Platelets& Pl, int precision, Control* ctl, cudaStream_t st) {
  const PlateletConst& k = Pl.k;
  const int PE = k.P * k.E;
  if (!k.morse || PE == 0) return cudaSuccess;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (!morse_uses_cells(k)) {
    const int slices = (k.E + 31) / 32;
    if (precision == PF_PREC_FP64) {
      platelet_bounds_k<double><<<k.P, kBoundsThreads, 0, st>>>(k, Pl.X, Pl.Y, Pl.Z, Pl.bounds, (D4*)Pl.relpos, ctl);
      const size_t smem = 2 * (size_t)k.E * sizeof(D4);
      cudaFuncSetAttribute(morse_platelet_k<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      morse_platelet_k<double><<<k.P * slices, 32 * kMorseSplit, smem, st>>>(k, Pl.bounds, (const D4*)Pl.relpos, slices,
                                                                Pl.Fmorse, ctl);
    } else {
      platelet_bounds_k<float><<<k.P, kBoundsThreads, 0, st>>>(k, Pl.X, Pl.Y, Pl.Z, Pl.bounds, (float4*)Pl.relpos, ctl);
      const size_t smem = 2 * (size_t)k.E * sizeof(float4);
      cudaFuncSetAttribute(morse_platelet_k<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      morse_platelet_k<float><<<k.P * slices, 32 * kMorseSplit, smem, st>>>(k, Pl.bounds, (const float4*)Pl.relpos, slices,
                                                               Pl.Fmorse, ctl);
    }
    return cudaGetLastError();
  }
  const int ncells = k.ncell[0] * k.ncell[1] * k.ncell[2];
  const unsigned grid = (unsigned)std::min(ncells, sms * 16);
  sort_bins_k<<<(unsigned)std::min(ncells, sms * 8), 256, 0, st>>>(ncells, Pl.bin_count, (float4*)Pl.bin, ctl);
  bool fast = precision != PF_PREC_FP64;
  for (int a = 0; a < 3; ++a)
    if (k.wrap[a] && k.ncell[a] < 3) fast = false;
  if (precision == PF_PREC_FP64)
    morse_k<double, false><<<grid, 128, 0, st>>>(k, Pl.X, Pl.Y, Pl.Z, Pl.bin_count, (const float4*)Pl.bin,
                                                 Pl.Fmorse, ctl);
  else if (fast)
    morse_k<float, true><<<grid, 128, 0, st>>>(k, Pl.X, Pl.Y, Pl.Z, Pl.bin_count, (const float4*)Pl.bin, Pl.Fmorse,
                                               ctl);
  else
    morse_k<float, false><<<grid, 128, 0, st>>>(k, Pl.X, Pl.Y, Pl.Z, Pl.bin_count, (const float4*)Pl.bin,
                                                Pl.Fmorse, ctl);
  return cudaGetLastError();
}

cudaError_t sort_cell_bins(Platelets& Pl, Control* ctl, cudaStream_t st) {
  const PlateletConst& k = Pl.k;
  if (!k.morse) return cudaSuccess;
  const int ncells = k.ncell[0] * k.ncell[1] * k.ncell[2];
  sort_bins_k<<<(unsigned)std::min(ncells, 1216), 256, 0, st>>>(ncells, Pl.bin_count, (float4*)Pl.bin, ctl);
  return cudaGetLastError();
}

cudaError_t fibrin_forces(Fibrin& Fb, int precision, Control* ctl, cudaStream_t st) {
  if (Fb.M == 0) return cudaSuccess;
  if (precision == PF_PREC_FP64)
    fibrin_k<double><<<(Fb.M + 127) / 128, 128, 0, st>>>(Fb.M, Fb.law, Fb.k, Fb.mass, Fb.X, Fb.Y, Fb.Z, Fb.ptr,
                                                         Fb.nbr, Fb.L0, Fb.F, ctl);
  else
    fibrin4_k<<<(unsigned)(((long long)Fb.M * kFibLanes + 127) / 128), 128, 0, st>>>(
        Fb.M, Fb.law, Fb.k, Fb.mass, Fb.X, Fb.Y, Fb.Z, Fb.ptr, Fb.nbr, Fb.L0, Fb.F, ctl);
  return cudaGetLastError();
}

// ------------------------------------------------ fibrin penalty coupling
// Flow at a fibrin node (fiber.cpp:753-814, its DH1D kernel restated as the
// IBM kernel the markers use): velocity (lattice units) and density summed
// with the stencil weights over the moments buffer, nodes of the Zou/He wall
// planes skipped, weights not renormalised.
template <class R>
__device__ __forceinline__ void fib_flow(const LatticeConst& lk, const R4<R>* ubuf, double x, double y, double z,
                                         double u[3], double& rho) {
  int nxa[5], nya[5], nza[5], rx[5], ry[5], rz[5];
  R wx[5], wy[5], wz[5];
  const int cxn = axis_stencil<R>(x, lk.dxf, lk.inv_dx, lk.nx, lk.ibm_wrap[0], 0, nxa, rx, wx);
  const int cyn = axis_stencil<R>(y, lk.dxf, lk.inv_dx, lk.ny, lk.ibm_wrap[1], 0, nya, ry, wy);
  const int czn = axis_stencil<R>(z, lk.dxf, lk.inv_dx, lk.nz, 0, 0, nza, rz, wz);
  const bool walls = lk.bc[2] == PF_BC_ZOUHE_SHEAR;
  R a0 = 0, a1 = 0, a2 = 0, r = 0;
  for (int c = 0; c < czn; ++c) {
    if (walls && (nza[c] == 0 || nza[c] == lk.nz - 1)) continue;
    for (int b = 0; b < cyn; ++b)
      for (int a = 0; a < cxn; ++a) {
        const R delta = wx[a] * wy[b] * wz[c];
        const size_t n = (size_t)nxa[a] + (size_t)lk.nx * ((size_t)nya[b] + (size_t)lk.ny * nza[c]);
        const R4<R> v = ubuf[n];
        a0 += v.y * delta; a1 += v.z * delta; a2 += v.w * delta;
        r += ((R)1 + v.x) * delta;
      }
  }
  u[0] = (double)a0; u[1] = (double)a1; u[2] = (double)a2;
  rho = (double)r;
}

// Node force kappa rho (u - V) (lattice units; V is kept in the element
// velocity units, V/C in lattice units) and its reaction for the next
// step's spreading, in reference force units (lattice force * F0 / kc).
template <class R>
__global__ void __launch_bounds__(128) fibrin_fsi_k(LatticeConst lk, int M, const double* X, const double* Y,
                                                    const double* Z, const double* V, const R4<R>* ubuf,
                                                    double kappa, double F0, double* Ffsi, double* Fs,
                                                    const Control* ctl) {
  if (ctl->done) return;
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  double u[3], rho;
  fib_flow<R>(lk, ubuf, X[m], Y[m], Z[m], u, rho);
  const double C = lk.C, kc = lk.kcoll;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double f = kappa * rho * (u[a] - V[(size_t)a * M + m] / C);
    Ffsi[(size_t)a * M + m] = f;
    Fs[(size_t)a * M + m] = -f / kc * F0;
  }
}

// network::solverkick (network.cpp:839-881) over half a lattice step on the
// node velocity in lattice units: v <- e^{-g/2} v + a (1 - e^{-g/2}) / g
// (a/2 for g = 0), a = (link force * kc / F0 + penalty force) / mass; fixed
// nodes rest.  Phase 0 then drifts the free nodes (the position update of
// the markers); phase 1 sets the occupancy bits of the next step.
__global__ void __launch_bounds__(128) fibrin_kick_k(LatticeConst lk, int M, int phase, double* X, double* Y,
                                                     double* Z, double* V, const int* fixed, const double* F,
                                                     const double* Ffsi, double F0, double mass, double gamma,
                                                     unsigned* mark, const Control* ctl, bool fp64) {
  if (ctl->done) return;
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  const double C = lk.C, kc = lk.kcoll;
  const double vdt = exp(-0.5 * gamma), fdt = gamma > 0 ? (1.0 - vdt) / gamma : 0.5;
  const bool fx = fixed[m] != 0;
  double v[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const size_t i = (size_t)a * M + m;
    if (fx) {
      v[a] = 0;
    } else {
      const double acc = (F[i] / F0 * kc + Ffsi[i]) / mass;
      v[a] = (vdt * (V[i] / C) + acc * fdt) * C;
    }
    V[i] = v[a];
  }
  double x = X[m], y = Y[m], z = Z[m];
  if (phase == 0) {
    if (fx) return;
    const float dtT = lk.dtT;
    const double Lx = lk.Lx, Ly = lk.Ly;
    x += v[0] * dtT;
    if (lk.ibm_wrap[0]) { if (x > Lx) x -= Lx; else if (x < 0) x += Lx; }
    y += v[1] * dtT;
    if (lk.ibm_wrap[1]) { if (y > Ly) y -= Ly; else if (y < 0) y += Ly; }
    z += v[2] * dtT;
    X[m] = x; Y[m] = y; Z[m] = z;
    return;
  }
  mark_node(lk, mark + (size_t)((int)(ctl->step & 1) ^ 1) * lk.nbricks, x, y, z, fp64);
}

template <class R>
__global__ void __launch_bounds__(128) fibrin_vinit_k(LatticeConst lk, int M, const double* X, const double* Y,
                                                      const double* Z, double* V, const int* fixed,
                                                      const R4<R>* ubuf) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  double u[3] = {0, 0, 0}, rho = 0;
  if (!fixed[m]) fib_flow<R>(lk, ubuf, X[m], Y[m], Z[m], u, rho);
  for (int a = 0; a < 3; ++a) V[(size_t)a * M + m] = u[a] * lk.C;
}

cudaError_t fibrin_penalty_step(Lattice& L, Fibrin& Fb, int precision, double F0, Control* ctl, cudaStream_t st) {
  if (Fb.M == 0) return cudaSuccess;
  const unsigned grid = (Fb.M + 127) / 128;
  const bool fp64 = precision == PF_PREC_FP64;
  if (fp64)
    fibrin_fsi_k<double><<<grid, 128, 0, st>>>(L.k, Fb.M, Fb.X, Fb.Y, Fb.Z, Fb.V, (const D4*)L.ubuf, Fb.kappa, F0,
                                               Fb.Ffsi, Fb.Fs, ctl);
  else
    fibrin_fsi_k<float><<<grid, 128, 0, st>>>(L.k, Fb.M, Fb.X, Fb.Y, Fb.Z, Fb.V, (const float4*)L.ubuf, Fb.kappa,
                                              F0, Fb.Ffsi, Fb.Fs, ctl);
  fibrin_kick_k<<<grid, 128, 0, st>>>(L.k, Fb.M, 0, Fb.X, Fb.Y, Fb.Z, Fb.V, Fb.fixed, Fb.F, Fb.Ffsi, Fb.f0,
                                      Fb.node_mass, Fb.gamma, L.mark, ctl, fp64);
  cudaError_t e = fibrin_forces(Fb, precision, ctl, st);
  if (e != cudaSuccess) return e;
  fibrin_kick_k<<<grid, 128, 0, st>>>(L.k, Fb.M, 1, Fb.X, Fb.Y, Fb.Z, Fb.V, Fb.fixed, Fb.F, Fb.Ffsi, Fb.f0,
                                      Fb.node_mass, Fb.gamma, L.mark, ctl, fp64);
  return cudaGetLastError();
}

cudaError_t fibrin_penalty_init(Lattice& L, Fibrin& Fb, cudaStream_t st) {
  if (Fb.M == 0) return cudaSuccess;
  const unsigned grid = (Fb.M + 127) / 128;
  if (L.precision == PF_PREC_FP64)
    fibrin_vinit_k<double><<<grid, 128, 0, st>>>(L.k, Fb.M, Fb.X, Fb.Y, Fb.Z, Fb.V, Fb.fixed, (const D4*)L.ubuf);
  else
    fibrin_vinit_k<float><<<grid, 128, 0, st>>>(L.k, Fb.M, Fb.X, Fb.Y, Fb.Z, Fb.V, Fb.fixed, (const float4*)L.ubuf);
  return cudaGetLastError();
}

cudaError_t bond_pass(Platelets& Pl, int precision, Control* ctl, cudaStream_t st) {
  const PlateletConst& k = Pl.k;
  const int NR = k.P * k.nrec;
  if (NR == 0) return cudaSuccess;
  RecTmp* tmp = (RecTmp*)Pl.rec_tmp;
  int* active = (int*)(tmp + NR);
  size_t ops_n = 1;
  while (ops_n < (size_t)2 * NR) ops_n <<= 1;
  unsigned long long* ops = (unsigned long long*)(((uintptr_t)(active + NR) + 15) & ~(uintptr_t)15);
  const int cap = 2 * NR;
  const int PE = k.P * k.E;
  const int fb = precision == PF_PREC_FP64 ? 8 : 4;
  const int threads = 256;
  int blocks = (NR + threads - 1) / threads;
  bonds_prepare_k<<<blocks, threads, 0, st>>>(k, Pl.X, Pl.Y, Pl.Z, Pl.tri, Pl.rec_tri, Pl.r1, Pl.r2, Pl.rec_state,
                                              tmp, active, ops, cap, Pl.Fbond, fb, ctl);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  (void)PE;
  if (precision == PF_PREC_FP64)
    bonds_resolve_k<double><<<1, 1024, 0, st>>>(k, Pl.X, Pl.Y, Pl.Z, Pl.tri, Pl.rec_tri, Pl.rec_state, Pl.vwf, tmp,
                                                active, ops, cap, (double*)Pl.Fbond, ctl);
  else
    bonds_resolve_k<float><<<1, 1024, 0, st>>>(k, Pl.X, Pl.Y, Pl.Z, Pl.tri, Pl.rec_tri, Pl.rec_state, Pl.vwf, tmp,
                                               active, ops, cap, (float*)Pl.Fbond, ctl);
  return cudaGetLastError();
}

size_t bond_scratch_bytes(int NR) {
  size_t ops = 1;
  while (ops < (size_t)2 * NR) ops <<= 1;
  return (size_t)NR * sizeof(RecTmp) + (size_t)NR * sizeof(int) + 16 + ops * sizeof(unsigned long long) + 64;
}

// Threads per CTA of the per-marker spreading and interpolation launches:
// one warp.  These kernels are bound by scattered L1/L2 accesses, not by
// warps; one-warp CTAs spread the markers evenly over the SMs (30,000
// elements make 235 CTAs of 128 threads, one or two per SM, but 938 of 32).
// Measured on the 256x128x128 channel: spreading 41.3 -> 39.3 us,
// interpolation 25.0 -> 24.3 us, the step 0.5 % faster than with 128.
static int marker_block() { return 32; }

cudaError_t spread_markers(Lattice& L, Platelets* Pl, Fibrin* Fb, Control* ctl, cudaStream_t st) {
  const int PE = Pl ? Pl->k.P * Pl->k.E : 0;
  const int M = Fb ? Fb->M : 0;
  if (PE + M == 0) return cudaSuccess;
  const unsigned grid = (PE + M + 127) / 128;
  const double F0 = Pl ? (double)Pl->k.f0 : 1.0;
  if (L.precision != PF_PREC_FP64 && !L.ibm_box)
    spread_k<float><<<grid, 128, 0, st>>>(
        L.k, (float4*)L.F[0], (float4*)L.F[1], PE, Pl ? Pl->X : nullptr, Pl ? Pl->Y : nullptr,
        Pl ? Pl->Z : nullptr, Pl ? (float*)Pl->Fmem : nullptr, (Pl && Pl->k.morse) ? Pl->Fmorse : nullptr,
        (Pl && Pl->k.nrec) ? (float*)Pl->Fbond : nullptr, Pl ? Pl->Ftot : nullptr, M, Fb ? Fb->X : nullptr,
        Fb ? Fb->Y : nullptr, Fb ? Fb->Z : nullptr, Fb ? Fb->spread_force() : nullptr, F0, ctl);
  else if (L.precision == PF_PREC_FP64)
    spread_k<double><<<grid, 128, 0, st>>>(
        L.k, (D4*)L.F[0], (D4*)L.F[1], PE, Pl ? Pl->X : nullptr,
        Pl ? Pl->Y : nullptr, Pl ? Pl->Z : nullptr, Pl ? (double*)Pl->Fmem : nullptr,
        (Pl && Pl->k.morse) ? Pl->Fmorse : nullptr, (Pl && Pl->k.nrec) ? (double*)Pl->Fbond : nullptr,
        Pl ? Pl->Ftot : nullptr, M, Fb ? Fb->X : nullptr, Fb ? Fb->Y : nullptr, Fb ? Fb->Z : nullptr,
        Fb ? Fb->spread_force() : nullptr, F0, ctl);
  else {
    // FP32: one CTA per platelet box, then the fibrin nodes
    cudaFuncSetAttribute(spread_box_k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBoxSmem);
    const int P = Pl ? Pl->k.P : 0, E = Pl ? Pl->k.E : 0;
    const unsigned g2 = (unsigned)(P + (M + kBoxFibrin - 1) / kBoxFibrin);
    spread_box_k<<<g2, kBoxThreads, (int)kBoxSmem, st>>>(
        L.k, (float4*)L.F[0], (float4*)L.F[1], P, E, Pl ? Pl->X : nullptr, Pl ? Pl->Y : nullptr,
        Pl ? Pl->Z : nullptr, Pl ? (float*)Pl->Fmem : nullptr, (Pl && Pl->k.morse) ? Pl->Fmorse : nullptr,
        (Pl && Pl->k.nrec) ? (float*)Pl->Fbond : nullptr, Pl ? Pl->Ftot : nullptr, M, Fb ? Fb->X : nullptr,
        Fb ? Fb->Y : nullptr, Fb ? Fb->Z : nullptr, Fb ? Fb->spread_force() : nullptr, F0, ctl);
  }
  return cudaGetLastError();
}

bool spread_split(const Lattice& L) { return L.precision != PF_PREC_FP64 && !L.ibm_box; }

// One force part: the markers, their positions and forces (Fa float, Fd
// double divided by div), one thread or four lanes per marker.
static cudaError_t launch_spread(const Lattice& L, int n, const double* X, const double* Y, const double* Z,
                                 const float* Fa, const double* Fd, double div, Control* ctl, cudaStream_t st) {
  const double rdiv = 1.0 / div;  // the device's FP64 quotient, rounded the same (IEEE)
  if (L.spread_lanes == kSpreadLanes) {
    const long long threads = (long long)n * kSpreadLanes;
    spread4_k<<<(unsigned)((threads + 127) / 128), 128, 0, st>>>(L.k, (float4*)L.F[0], (float4*)L.F[1], n, X, Y, Z,
                                                                  Fa, Fd, rdiv, ctl);
  } else {
    spread_part_k<<<(n + marker_block() - 1) / marker_block(), marker_block(), 0, st>>>(
        L.k, (float4*)L.F[0], (float4*)L.F[1], n, X, Y, Z, Fa, Fd, rdiv, ctl);
  }
  return cudaGetLastError();
}

cudaError_t spread_part(Lattice& L, Platelets* Pl, Fibrin* Fb, Control* ctl, int part, cudaStream_t st) {
  if (part == 2) {
    if (!Fb || Fb->M == 0) return cudaSuccess;
    const double F0 = Pl ? (double)Pl->k.f0 : 1.0;
    return launch_spread(L, Fb->M, Fb->X, Fb->Y, Fb->Z, nullptr, Fb->spread_force(), F0, ctl, st);
  }
  const int PE = Pl ? Pl->k.P * Pl->k.E : 0;
  if (PE == 0 || (part == 1 && !Pl->k.nrec)) return cudaSuccess;
  const float* Fa = (const float*)(part == 0 ? Pl->Fmem : Pl->Fbond);
  const double* Fd = part == 0 && Pl->k.morse ? Pl->Fmorse : nullptr;
  return launch_spread(L, PE, Pl->X, Pl->Y, Pl->Z, Fa, Fd, 1.0, ctl, st);
}

cudaError_t mark_markers(Lattice& L, Platelets* Pl, Fibrin* Fb, cudaStream_t st) {
  const int PE = Pl ? Pl->k.P * Pl->k.E : 0;
  const int M = Fb ? Fb->M : 0;
  if (PE + M == 0) return cudaSuccess;
  mark_markers_k<<<(PE + M + 127) / 128, 128, 0, st>>>(L.k, L.mark, PE, Pl ? Pl->X : nullptr, Pl ? Pl->Y : nullptr,
                                                       Pl ? Pl->Z : nullptr, M, Fb ? Fb->X : nullptr,
                                                       Fb ? Fb->Y : nullptr, Fb ? Fb->Z : nullptr,
                                                       L.precision == PF_PREC_FP64);
  return cudaGetLastError();
}

cudaError_t flag_markers(Lattice& L, Platelets* Pl, Fibrin* Fb, Control* ctl, cudaStream_t st, bool check_near,
                         bool with_prev) {
  const int PE = Pl ? Pl->k.P * Pl->k.E : 0;
  const int M = Fb ? Fb->M : 0;
  if (PE + M == 0) return cudaSuccess;
  const int R = flag_rows(L.k.nbx);
  if ((R + 2 * kFlagR) * L.k.nbx > kFlagWords) return cudaErrorInvalidValue;  // rows wider than 131072 nodes
  flag_k<<<L.k.nz * ((L.k.ny + R - 1) / R), kFlagThreads, 0, st>>>(L.k, L.mark, L.flags[0], L.flags[1], L.list[0], L.list[1],
                                           check_near ? L.near[0] : nullptr, check_near ? L.near[1] : nullptr,
                                           L.precision == PF_PREC_FP64 ? kFlagR : kFlagR - 1, ctl, with_prev);
  return cudaGetLastError();
}

cudaError_t interp_advance(Lattice& L, Platelets* Pl, Fibrin* Fb, Control* ctl, double detach_rate,
                           uint64_t seed, unsigned* done_blocks, cudaStream_t st) {
  const int PE = Pl ? Pl->k.P * Pl->k.E : 0;
  const int M = Fb ? Fb->M : 0;
  const int mb = marker_block();
  const unsigned grid = (PE + M + mb - 1) / mb > 0 ? (PE + M + mb - 1) / mb : 1;
  PlateletConst pk{};
  if (Pl) pk = Pl->k;
  // elements are binned every step only when the Morse pass uses the cell list
  const bool cells = Pl && Pl->k.morse && morse_uses_cells(Pl->k);
  int* bc = cells ? Pl->bin_count : nullptr;
  float4* bn = cells ? (float4*)Pl->bin : nullptr;
  if (L.precision == PF_PREC_FP64)
    interp_advance_k<double><<<grid, mb, 0, st>>>(
        L.k, pk, (const D4*)L.ubuf, PE, Pl ? Pl->X : nullptr, Pl ? Pl->Y : nullptr, Pl ? Pl->RY : nullptr,
        Pl ? Pl->Z : nullptr, Pl ? Pl->V : nullptr, M, Fb ? Fb->X : nullptr, Fb ? Fb->Y : nullptr,
        Fb ? Fb->Z : nullptr, Fb ? Fb->V : nullptr, Fb ? Fb->fixed : nullptr, bc, bn, L.mark, ctl, done_blocks,
        detach_rate, seed, nullptr, nullptr, nullptr, nullptr);
  else if (PE + M == 0 || !L.ibm_box) {
    interp_advance_k<float><<<grid, mb, 0, st>>>(
        L.k, pk, (const float4*)L.ubuf, PE, Pl ? Pl->X : nullptr, Pl ? Pl->Y : nullptr, Pl ? Pl->RY : nullptr,
        Pl ? Pl->Z : nullptr, Pl ? Pl->V : nullptr, M, Fb ? Fb->X : nullptr, Fb ? Fb->Y : nullptr,
        Fb ? Fb->Z : nullptr, Fb ? Fb->V : nullptr, Fb ? Fb->fixed : nullptr, bc, bn, L.mark, ctl, done_blocks,
        detach_rate, seed, Pl ? (const float*)Pl->Fmem : nullptr, (Pl && Pl->k.morse) ? Pl->Fmorse : nullptr,
        (Pl && Pl->k.nrec) ? (const float*)Pl->Fbond : nullptr, Pl ? Pl->Ftot : nullptr);
  } else {
    cudaFuncSetAttribute(interp_box_k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBoxSmem);
    const int P = Pl ? Pl->k.P : 0, E = Pl ? Pl->k.E : 0;
    const unsigned g2 = (unsigned)(P + (M + kBoxFibrin - 1) / kBoxFibrin);
    interp_box_k<<<g2, kBoxThreads, (int)kBoxSmem, st>>>(
        L.k, pk, (const float4*)L.ubuf, P, E, Pl ? Pl->X : nullptr, Pl ? Pl->Y : nullptr, Pl ? Pl->RY : nullptr,
        Pl ? Pl->Z : nullptr, Pl ? Pl->V : nullptr, M, Fb ? Fb->X : nullptr, Fb ? Fb->Y : nullptr,
        Fb ? Fb->Z : nullptr, Fb ? Fb->V : nullptr, Fb ? Fb->fixed : nullptr, bc, bn, L.mark, ctl, done_blocks,
        detach_rate, seed);
  }
  return cudaGetLastError();
}

cudaError_t bin_elements(Platelets& Pl, Control* ctl, cudaStream_t st) {
  const int PE = Pl.k.P * Pl.k.E;
  if (!Pl.k.morse || PE == 0) return cudaSuccess;
  cudaMemsetAsync(Pl.bin_count, 0, sizeof(int) * (size_t)Pl.ncells, st);
  cudaMemsetAsync(&ctl->occupied, 0, sizeof(int), st);
  bin_elements_k<<<(PE + 127) / 128, 128, 0, st>>>(Pl.k, PE, Pl.X, Pl.Y, Pl.Z, Pl.bin_count, (float4*)Pl.bin, ctl);
  return cudaGetLastError();
}


bool batch_supported(const BatchDesc& d) {
  // the flag kernel stages whole rows (plus halo) of a plane in shared memory
  return (flag_rows(d.L.k.nbx) + 2 * kFlagR) * d.L.k.nbx <= kFlagWords;
}

int batch_threads(int kind, const BatchTune& t) {
  switch (kind) {
    case BK_FLAG: return kFlagThreads;
    case BK_MEMBRANE: return kMem32Threads;
    case BK_BOUNDS: return kBoundsThreads;
    case BK_MORSE: return 32 * kMorseSplit;
    case BK_BOND_PREP: return 256;
    case BK_BOND_RESOLVE: return 1024;
    case BK_LBM_UNFLAGGED: case BK_LBM_FLAGGED: case BK_MOMENTS: return kLbmBlock;
    default: return t.marker_threads;
  }
}

size_t batch_smem(const BatchDesc& d, int kind) {
  if (!d.has_pl) return 0;
  if (kind == BK_MEMBRANE) return Mem32Layout(d.Pl.k).bytes;
  if (kind == BK_MORSE) return 2 * (size_t)d.Pl.k.E * sizeof(float4);
  return 0;
}

int batch_ctas(const BatchDesc& d, int kind, int sms, int njobs, const BatchTune& t) {
  const LatticeConst& lk = d.L.k;
  const PlateletConst& pk = d.Pl.k;
  const int PE = d.has_pl ? pk.P * pk.E : 0;
  const int M = d.has_fb ? d.Fb.M : 0;
  const int NR = d.has_pl ? pk.P * pk.nrec : 0;
  const bool markers = PE + M > 0;
  switch (kind) {
    case BK_FLAG: {
      if (!markers) return 0;
      const int R = flag_rows(lk.nbx);
      return lk.nz * ((lk.ny + R - 1) / R);
    }
    case BK_LBM_UNFLAGGED:
      return ((lk.nbricks + kLbmBlock / kBrickX - 1) / (kLbmBlock / kBrickX) + t.lbm_rows - 1) / t.lbm_rows;
    case BK_MEMBRANE: return PE ? pk.P : 0;
    case BK_BOUNDS: return PE && pk.morse ? pk.P : 0;
    case BK_MORSE: return PE && pk.morse ? pk.P * ((pk.E + 31) / 32) : 0;
    case BK_BOND_PREP: return NR ? (NR + 255) / 256 : 0;
    case BK_BOND_RESOLVE: return NR ? 1 : 0;
    case BK_FIBRIN: return M ? (M + t.marker_threads - 1) / t.marker_threads : 0;
    case BK_SPREAD_ELEM: return PE ? (kSpreadLanes * PE + t.marker_threads - 1) / t.marker_threads : 0;
    case BK_SPREAD_BOND: return PE && pk.nrec ? (kSpreadLanes * PE + t.marker_threads - 1) / t.marker_threads : 0;
    case BK_SPREAD_FIB: return M ? (kSpreadLanes * M + t.marker_threads - 1) / t.marker_threads : 0;
    case BK_LBM_FLAGGED:
    case BK_MOMENTS: {
      if (!markers) return 0;
      const int need = (lk.nbricks + kLbmBlock / 32 - 1) / (kLbmBlock / 32);
      const int cap = std::max(8, (sms * t.list_per_sm + njobs - 1) / std::max(1, njobs));
      return std::min(need, cap);
    }
    case BK_INTERP: return std::max(1, (PE + M + t.marker_threads - 1) / t.marker_threads);
  }
  return 0;
}

cudaError_t batch_launch(int kind, const BatchDesc* descs, const int* start, int nj, int total, size_t smem,
                         int precision, bool fast, const BatchTune& t, cudaStream_t st) {
  if (total <= 0) return cudaSuccess;
  const int mt = t.marker_threads;
  if (mt < 32 || mt > kMarkerThreadsMax || mt % 32) return cudaErrorInvalidValue;
  switch (kind) {
    case BK_LBM_UNFLAGGED: case BK_LBM_FLAGGED: case BK_MOMENTS:
      return batch_launch_lattice(kind, descs, start, nj, total, precision, fast, t.lbm_rows, st);
    case BK_FLAG: flag_batch_k<<<total, kFlagThreads, 0, st>>>(descs, start, nj); break;
    case BK_MEMBRANE: {
      cudaError_t e = cudaFuncSetAttribute(membrane_batch_k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)kMem32MaxSmem);
      if (e != cudaSuccess) return e;
      membrane_batch_k<<<total, kMem32Threads, smem, st>>>(descs, start, nj);
      break;
    }
    case BK_BOUNDS: bounds_batch_k<<<total, kBoundsThreads, 0, st>>>(descs, start, nj); break;
    case BK_MORSE:
      cudaFuncSetAttribute(morse_batch_k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      morse_batch_k<<<total, 32 * kMorseSplit, smem, st>>>(descs, start, nj);
      break;
    case BK_BOND_PREP: bond_prep_batch_k<<<total, 256, 0, st>>>(descs, start, nj); break;
    case BK_BOND_RESOLVE: bond_resolve_batch_k<<<total, 1024, 0, st>>>(descs, start, nj); break;
    case BK_FIBRIN: fibrin_batch_k<<<total, mt, 0, st>>>(descs, start, nj); break;
    case BK_SPREAD_ELEM: spread_batch_k<0><<<total, mt, 0, st>>>(descs, start, nj); break;
    case BK_SPREAD_BOND: spread_batch_k<1><<<total, mt, 0, st>>>(descs, start, nj); break;
    case BK_SPREAD_FIB: spread_batch_k<2><<<total, mt, 0, st>>>(descs, start, nj); break;
    case BK_INTERP: interp_batch_k<<<total, mt, 0, st>>>(descs, start, nj); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace pf
