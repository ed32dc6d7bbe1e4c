// pf_lattice.cu -- D3Q19 lattice kernels: the fused pull-scheme
// collide-stream step with boundary conditions, moments on active bricks,
// upload (un-streaming) and download.
//
// Reference semantics kept (LB_kernel.cu): the collision of step t uses the
// density/velocity of step t-1 (moments of fIN with the half force of step
// t-1, :1108-1199) and the force of step t (:1203-1304); streaming is
// periodic on every axis (:1312-1359) and the Zou/He planes then overwrite
// the five unknown populations (:395-780), where density and velocity are the
// boundary values (those planes are obstacle nodes for the moments kernel).
// Arithmetic is in lattice units on shifted populations g = f - w:
//   geq_d = w_d (drho + rho (3 c.u + 4.5 (c.u)^2 - 1.5 u.u))
//   S_d   = w_d (1 - omega/2) (3 c.F + 9 (c.u)(c.F) - 3 u.F)
// which is the reference's Guo forcing with u -> u/C and F -> F*K*dt/C.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "pf_internal.h"

namespace pf {

namespace {

// weight class of a direction (rest, axis, diagonal): index of the FP16
// store scales w_d * sigma and their inverses in LatticeConst
__host__ __device__ constexpr int wcls(int d) { return d == 0 ? 0 : (d < 7 ? 1 : 2); }

// a lattice constant in the arithmetic type: the double, or its float
// rounding stored beside it
template <class R>
__device__ __forceinline__ R kv(double d, float f) {
  if constexpr (sizeof(R) == 4) return f;
  else return (R)d;
}

template <class S, class R>
__device__ __forceinline__ R ld(const S* p, int d, const LatticeConst& k) {
  return (R)StoreTraits<S>::load(p, d, (decltype(StoreTraits<S>::load(p, 0, R(0))))k.hs[wcls(d)]);
}
template <class S, class R>
__device__ __forceinline__ void st(S* p, R v, int d, const LatticeConst& k) {
  StoreTraits<S>::store(p, v, d, (decltype(StoreTraits<S>::load(p, 0, R(0))))k.hinv[wcls(d)]);
}

template <class R>
__device__ __forceinline__ void ld_force(const R4<R>* F, size_t n, R& fx, R& fy, R& fz);
template <>
__device__ __forceinline__ void ld_force<float>(const float4* F, size_t n, float& fx, float& fy, float& fz) {
  float4 v = __ldcg(F + n);
  fx += v.x; fy += v.y; fz += v.z;
}
template <>
__device__ __forceinline__ void ld_force<double>(const D4* F, size_t n, double& fx, double& fy, double& fz) {
  const double2* p = reinterpret_cast<const double2*>(F + n);
  double2 a = __ldcg(p), b = __ldcg(p + 1);
  fx += a.x; fy += a.y; fz += b.x;
}
template <class R>
__device__ __forceinline__ void zero_force(R4<R>* F, size_t n);
template <>
__device__ __forceinline__ void zero_force<float>(float4* F, size_t n) { F[n] = make_float4(0, 0, 0, 0); }
template <>
__device__ __forceinline__ void zero_force<double>(D4* F, size_t n) { F[n] = D4{0, 0, 0, 0}; }

template <class R>
__device__ __forceinline__ void st_u(R4<R>* U, size_t n, R a, R b, R c, R d);
template <>
__device__ __forceinline__ void st_u<float>(float4* U, size_t n, float a, float b, float c, float d) {
  U[n] = make_float4(a, b, c, d);
}
template <>
__device__ __forceinline__ void st_u<double>(D4* U, size_t n, double a, double b, double c, double d) {
  U[n] = D4{a, b, c, d};
}
template <class R>
__device__ __forceinline__ void ld_u(const R4<R>* U, size_t n, R& a, R& b, R& c, R& d);
template <>
__device__ __forceinline__ void ld_u<float>(const float4* U, size_t n, float& a, float& b, float& c, float& d) {
  float4 v = U[n];
  a = v.x; b = v.y; c = v.z; d = v.w;
}
template <>
__device__ __forceinline__ void ld_u<double>(const D4* U, size_t n, double& a, double& b, double& c, double& d) {
  D4 v = U[n];
  a = v.x; b = v.y; c = v.z; d = v.w;
}

// Pull the 19 post-stream populations of node (x,y,z) from the post-collision
// buffer: periodic on periodic and Zou/He axes (the reference streams
// periodically first), half-way bounce-back through faces of bounce-back axes.
// RAW: the stored values as they are (FP16: q, not scaled back to g)
template <class S, class R, bool RAW>
__device__ __forceinline__ R ldr(const S* p, int d, const LatticeConst& k) {
  if constexpr (RAW && std::is_same<S, __half>::value) return __half2float(__ldg(p));
  else return ld<S, R>(p, d, k);
}

template <class S, class R, bool RAW = false>
__device__ __forceinline__ void gather(const LatticeConst& k, const S* __restrict__ gin, int x, int y, int z,
                                       R g[Q]) {
  const int nx = k.nx, ny = k.ny, nz = k.nz;
  const size_t N = (size_t)k.N;
  int xm = x - 1, xp = x + 1, ym = y - 1, yp = y + 1, zm = z - 1, zp = z + 1;
  bool oxm = false, oxp = false, oym = false, oyp = false, ozm = false, ozp = false;
  if (xm < 0) { if (k.bc[0] == PF_BC_BOUNCEBACK) oxm = true; else xm = nx - 1; }
  if (xp >= nx) { if (k.bc[0] == PF_BC_BOUNCEBACK) oxp = true; else xp = 0; }
  if (ym < 0) { if (k.bc[1] == PF_BC_BOUNCEBACK) oym = true; else ym = ny - 1; }
  if (yp >= ny) { if (k.bc[1] == PF_BC_BOUNCEBACK) oyp = true; else yp = 0; }
  if (zm < 0) { if (k.bc[2] == PF_BC_BOUNCEBACK) ozm = true; else zm = nz - 1; }
  if (zp >= nz) { if (k.bc[2] == PF_BC_BOUNCEBACK) ozp = true; else zp = 0; }
  const size_t n = (size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * z);
#pragma unroll
  for (int d = 0; d < Q; ++d) {
    const int sx = cx(d) == 1 ? xm : (cx(d) == -1 ? xp : x);
    const int sy = cy(d) == 1 ? ym : (cy(d) == -1 ? yp : y);
    const int sz = cz(d) == 1 ? zm : (cz(d) == -1 ? zp : z);
    const bool out = (cx(d) == 1 && oxm) || (cx(d) == -1 && oxp) || (cy(d) == 1 && oym) ||
                     (cy(d) == -1 && oyp) || (cz(d) == 1 && ozm) || (cz(d) == -1 && ozp);
    if (out) {
      g[d] = ldr<S, R, RAW>(gin + (size_t)opp(d) * N + n, opp(d), k);
    } else {
      g[d] = ldr<S, R, RAW>(gin + (size_t)d * N + (size_t)sx + (size_t)nx * ((size_t)sy + (size_t)ny * sz), d, k);
    }
  }
}

// The same pull for lattices without bounce-back faces (every axis periodic
// or Zou/He, which streams periodically) whose population index 19 N fits
// 32 bits: no face tests, 32-bit offsets (nine source rows, three columns).
template <class S, class R, bool RAW = false>
__device__ __forceinline__ void gather_fast(const LatticeConst& k, const S* __restrict__ gin, int x, int y, int z,
                                            R g[Q]) {
  const unsigned nx = (unsigned)k.nx, ny = (unsigned)k.ny, nz = (unsigned)k.nz;
  const unsigned N = (unsigned)k.N;
  const unsigned xs[3] = {x == 0 ? nx - 1 : (unsigned)x - 1, (unsigned)x, (unsigned)x + 1 == nx ? 0u : x + 1u};
  const unsigned ys[3] = {y == 0 ? ny - 1 : (unsigned)y - 1, (unsigned)y, (unsigned)y + 1 == ny ? 0u : y + 1u};
  const unsigned zs[3] = {z == 0 ? nz - 1 : (unsigned)z - 1, (unsigned)z, (unsigned)z + 1 == nz ? 0u : z + 1u};
#pragma unroll
  for (int d = 0; d < Q; ++d) {
    // pull from x - c: index 0 of each triple is the -1 neighbour
    const unsigned off = (unsigned)d * N + xs[1 - cx(d)] + nx * (ys[1 - cy(d)] + ny * zs[1 - cz(d)]);
    g[d] = ldr<S, R, RAW>(gin + off, d, k);
  }
}

// Zou/He planes: z=0 no-slip (LB_kernel.cu:395-600) and z=nz-1 moving plate
// (:602-780, where C, Nzx, Nzy are float).  Writes the unknowns, returns the
// boundary density; velocity is the wall's.
// Both return drho = rho - 1: in shifted form the weights of the summed
// populations add up to one.
template <class R>
__device__ __forceinline__ R zouhe_bottom(R g[Q]) {
  const R drho = (g[1] + g[2] + g[3] + g[4] + g[7] + g[8] + g[11] + g[12] + g[0] +
                  (R)2 * (g[6] + g[10] + g[14] + g[16] + g[18]));
  const R Nzx = (R)0.5 * (g[1] + g[7] + g[8] - g[2] - g[11] - g[12]);
  const R Nzy = (R)0.5 * (g[3] + g[7] + g[11] - g[4] - g[8] - g[12]);
  g[5] = g[6];
  g[9] = g[14] - Nzx;
  g[13] = g[10] + Nzx;
  g[15] = g[18] - Nzy;
  g[17] = g[16] + Nzy;
  return drho;
}
template <class R>
__device__ __forceinline__ R zouhe_top(R g[Q], R uw) {
  const R drho = (g[1] + g[2] + g[3] + g[4] + g[7] + g[11] + g[12] + g[8] + g[0] +
                  (R)2 * (g[5] + g[9] + g[13] + g[15] + g[17]));
  const R rho = (R)1 + drho;
  const R Nzx = (R)(float)((R)0.5 * (g[1] + g[7] + g[8] - g[2] - g[11] - g[12]));
  const R Nzy = (R)(float)((R)0.5 * (g[3] + g[7] + g[11] - g[4] - g[8] - g[12]) - (R)(1.0 / 3.0) * rho * uw);
  g[6] = g[5];
  g[10] = g[13] - Nzx;
  g[14] = g[9] + Nzx;
  g[16] = g[17] + (R)(1.0 / 6.0) * rho * uw - Nzy;
  g[18] = g[15] + (R)(1.0 / 6.0) * rho * (-uw) + Nzy;
  return drho;
}

// Velocity inlet (y=0) / outlet (y=ny-1) of LB_kernel.cu:78-392 at an
// interior node (0 < x < nx-1, 0 < z < nz-1) of those planes, on shifted
// populations in lattice units: u = (0, uw z/(nz-1), 0).  Rows next to the
// plane's edges: the equilibrium at unit density (the reference's
// re-initialisation).  Elsewhere Zou/He: the density from the in-plane and
// outgoing populations (their weights add up to one, so
// rho = (1 + G) / (1 -+ uy)), the unknowns from their opposites plus the
// momentum terms and the transverse corrections Nyx, Nyz.  Two slips of the
// reference's text are corrected: the inlet's f11 is built from f8 (the
// text reads f9), and the outlet computes its own Nyx, Nyz (the text uses
// values set only on the inlet branch).  The moments of the node are then
// taken from these populations as everywhere else.
template <class R>
__device__ __forceinline__ void inout_y(const LatticeConst& k, R g[Q], int x, int y, int z) {
  const R uy = kv<R>(k.uw, k.uw_f) * (R)z / (R)(k.nz - 1);
  if (x == 1 || x == k.nx - 2 || z == 1 || z == k.nz - 2) {
    const R usq = uy * uy;
#pragma unroll
    for (int d = 0; d < Q; ++d) {
      const R cu = (R)cy(d) * uy;
      g[d] = (R)wgt(d) * ((R)3 * cu + (R)4.5 * cu * cu - (R)1.5 * usq);
    }
    return;
  }
  const R inplane = g[1] + g[2] + g[5] + g[6] + g[9] + g[10] + g[13] + g[14] + g[0];
  const R Nyx = (R)0.5 * (g[1] + g[9] + g[10] - g[2] - g[13] - g[14]);
  const R Nyz = (R)0.5 * (g[5] + g[9] + g[13] - g[6] - g[10] - g[14]);
  if (y == 0) {
    const R rho = ((R)1 + inplane + (R)2 * (g[4] + g[8] + g[12] + g[17] + g[18])) / ((R)1 - uy);
    g[3] = g[4] + (R)(1.0 / 3.0) * rho * uy;
    g[7] = g[12] + (R)(1.0 / 6.0) * rho * uy - Nyx;
    g[11] = g[8] + (R)(1.0 / 6.0) * rho * uy + Nyx;
    g[15] = g[18] + (R)(1.0 / 6.0) * rho * uy - Nyz;
    g[16] = g[17] + (R)(1.0 / 6.0) * rho * uy + Nyz;
  } else {
    const R rho = ((R)1 + inplane + (R)2 * (g[3] + g[7] + g[11] + g[15] + g[16])) / ((R)1 + uy);
    g[4] = g[3] - (R)(1.0 / 3.0) * rho * uy;
    g[12] = g[7] - (R)(1.0 / 6.0) * rho * uy + Nyx;
    g[8] = g[11] - (R)(1.0 / 6.0) * rho * uy - Nyx;
    g[18] = g[15] - (R)(1.0 / 6.0) * rho * uy + Nyz;
    g[17] = g[16] - (R)(1.0 / 6.0) * rho * uy - Nyz;
  }
}

template <class R>
__device__ __forceinline__ void moments(const R g[Q], R& drho, R& jx, R& jy, R& jz) {
  drho = 0; jx = 0; jy = 0; jz = 0;
#pragma unroll
  for (int d = 0; d < Q; ++d) {
    drho += g[d];
    if (cx(d)) jx += cx(d) * g[d];
    if (cy(d)) jy += cy(d) * g[d];
    if (cz(d)) jz += cz(d) * g[d];
  }
}

// density deviation drho = rho - 1 and lattice velocity of a post-stream node
// (boundary values on the Zou/He planes, half-force corrected moments
// elsewhere).  drho is carried separately: rounding 1 + drho in FP32 would
// put ~6e-8 of noise into the density every step.
// Whether linear node n of plane z is an interior node of an inflow/outflow
// plane.
__device__ __forceinline__ bool on_inout(const LatticeConst& k, size_t n, int z) {
  if (k.bc[1] != PF_BC_INOUT || z == 0 || z == k.nz - 1) return false;
  const int y = (int)((n / (size_t)k.nx) % (size_t)k.ny);
  if (y != 0 && y != k.ny - 1) return false;
  const int x = (int)(n % (size_t)k.nx);
  return x > 0 && x < k.nx - 1;
}
template <class R>
__device__ __forceinline__ void node_state(const LatticeConst& k, R g[Q], int z, size_t n, bool apply_bc, R Fx,
                                           R Fy, R Fz, R& drho, R& ux, R& uy, R& uz) {
  if (apply_bc && on_inout(k, n, z))
    inout_y<R>(k, g, (int)(n % (size_t)k.nx), (int)((n / (size_t)k.nx) % (size_t)k.ny), z);
  if (apply_bc && k.bc[2] == PF_BC_ZOUHE_SHEAR && z == 0) {
    drho = zouhe_bottom(g);
    ux = 0; uy = 0; uz = 0;
    return;
  }
  if (apply_bc && k.bc[2] == PF_BC_ZOUHE_SHEAR && z == k.nz - 1) {
    drho = zouhe_top(g, kv<R>(k.uw, k.uw_f));
    ux = 0; uy = kv<R>(k.uw, k.uw_f); uz = 0;
    return;
  }
  R jx, jy, jz;
  moments(g, drho, jx, jy, jz);
  const R rho = (R)1 + drho;
  const R hk = (R)0.5 * kv<R>(k.kmom, k.kmom_f);
  ux = (jx + hk * Fx) / rho;
  uy = (jy + hk * Fy) / rho;
  uz = (jz + hk * Fz) / rho;
}

// c_d . (a, b, c) from the nonzero components only, in x, y, z order: the
// products with zero components of the term-by-term form cannot be folded
// away under IEEE rules (0 * x is not 0 for every x) and cost an FMA each.
// Equal to the term-by-term sum except for the sign of a zero result.
template <class R>
__device__ __forceinline__ R cdot(int d, R a, R b, R c) {
  R r = (R)0;
  bool any = false;
  if (cx(d) != 0) { r = cx(d) > 0 ? a : -a; any = true; }
  if (cy(d) != 0) { r = any ? (cy(d) > 0 ? r + b : r - b) : (cy(d) > 0 ? b : -b); any = true; }
  if (cz(d) != 0) { r = any ? (cz(d) > 0 ? r + c : r - c) : (cz(d) > 0 ? c : -c); }
  return r;
}

// BGK collision with Guo forcing of one node, in place on the shifted
// populations (F already scaled to lattice units, om = 1/tau, sf = 1 - om/2):
//   g_d <- g_d - om (g_d - geq_d) + S_d.
// FP64: term by term as written.  FP32: the same polynomial regrouped as
//   g_d <- (1 - om) g_d + w_d (A + B cu + C cu^2 + D cF + E cu cF)
// with per-node coefficients, evaluated once per opposite pair (d, opp d),
// whose cu and cF differ only in sign.
template <class R>
__device__ __forceinline__ void collide(R g[Q], R drho, R ux, R uy, R uz, R Fx, R Fy, R Fz, R om, R sf) {
  const R rho = (R)1 + drho;
  const R usq = ux * ux + uy * uy + uz * uz;
  const R uF = ux * Fx + uy * Fy + uz * Fz;
  if constexpr (sizeof(R) == 8) {
#pragma unroll
    for (int d = 0; d < Q; ++d) {
      const R cu = (R)cx(d) * ux + (R)cy(d) * uy + (R)cz(d) * uz;
      const R cF = (R)cx(d) * Fx + (R)cy(d) * Fy + (R)cz(d) * Fz;
      const R w = (R)wgt(d);
      const R geq = w * (drho + rho * ((R)3 * cu + (R)4.5 * cu * cu - (R)1.5 * usq));
      const R src = w * sf * ((R)3 * cF + (R)9 * cu * cF - (R)3 * uF);
      g[d] = g[d] - om * (g[d] - geq) + src;
    }
  } else {
    const R omr = om * rho;
    const R A = om * drho - (R)1.5 * omr * usq - (R)3 * sf * uF;
    const R B = (R)3 * omr, C = (R)4.5 * omr, D = (R)3 * sf, E = (R)9 * sf;
    const R omc = (R)1 - om;
    g[0] = omc * g[0] + (R)wgt(0) * A;
#pragma unroll
    for (int d = 1; d < Q; ++d) {
      if (opp(d) < d) continue;  // handled with its partner
      const int o = opp(d);
      const R cu = cdot<R>(d, ux, uy, uz);
      const R cF = cdot<R>(d, Fx, Fy, Fz);
      const R even = A + cu * (C * cu + E * cF);
      const R odd = B * cu + D * cF;
      const R w = (R)wgt(d);
      g[d] = omc * g[d] + w * (even + odd);
      g[o] = omc * g[o] + w * (even - odd);
    }
  }
}

// FP32 collision of a node without any force: collide's regrouped
// polynomial without the force terms (exact zeros there).
__device__ __forceinline__ void collide_noforce(float g[Q], float drho, float ux, float uy, float uz, float om) {
  const float rho = 1.0f + drho;
  const float usq = ux * ux + uy * uy + uz * uz;
  const float omr = om * rho;
  const float A = om * drho - 1.5f * omr * usq;
  const float B = 3.0f * omr, C = 4.5f * omr;
  const float omc = 1.0f - om;
  g[0] = omc * g[0] + (float)wgt(0) * A;
#pragma unroll
  for (int d = 1; d < Q; ++d) {
    if (opp(d) < d) continue;
    const int o = opp(d);
    const float cu = cdot<float>(d, ux, uy, uz);
    const float even = A + cu * (C * cu);
    const float odd = B * cu;
    const float w = (float)wgt(d);
    g[d] = omc * g[d] + w * (even + odd);
    g[o] = omc * g[o] + w * (even - odd);
  }
}

// The collision of one node with the step's force F = body + Fc.  FP32 nodes
// without any (no marker force, no body force) take collide_noforce; every
// FP32 kernel makes the same choice, so that they stay equal bit for bit.
template <typename R>
__device__ __forceinline__ void collide_node(const LatticeConst& k, R g[Q], R drho, R ux, R uy, R uz,
                                             const R4<R>* Fc, size_t n, unsigned fc, R kc, R om) {
  if constexpr (sizeof(R) == 4) {
    if (!fc && k.nobody) {
      collide_noforce(g, drho, ux, uy, uz, om);
      return;
    }
  }
  R Fx = kv<R>(k.body[0], k.body_f[0]), Fy = kv<R>(k.body[1], k.body_f[1]), Fz = kv<R>(k.body[2], k.body_f[2]);
  if (fc) ld_force<R>(Fc, n, Fx, Fy, Fz);
  collide<R>(g, drho, ux, uy, uz, Fx * kc, Fy * kc, Fz * kc, om, (R)1 - (R)0.5 * om);
}

// One node of the step on the FP16 store's own values q = g / (w_c sigma)
// (c: the weight class), in place.  Interior nodes: the moments from
// per-class sums (g = w_c sigma q) and the FP32 collision's polynomial with
// the weight folded into 1 / sigma,
//   q_d <- (1 - om) q_d + (A + B cu + C cu^2 + D cF + E cu cF) / sigma,
// so no per-population scaling on load or store.  The Zou/He planes go
// through g with the boundary pass of node_state.
__device__ __forceinline__ void node_q(const LatticeConst& k, float q[Q], int z, int first, size_t n,
                                       const float4* ubuf, const float4* Fp, unsigned fp, const float4* Fc,
                                       unsigned fc) {
  const float om = k.omega_f, sf = 1.0f - 0.5f * om, kc = k.kcoll_f;
  float Fx = k.body_f[0], Fy = k.body_f[1], Fz = k.body_f[2];
  if (fc) ld_force<float>(Fc, n, Fx, Fy, Fz);
  Fx *= kc; Fy *= kc; Fz *= kc;
  float drho, ux, uy, uz;
  if ((k.bc[2] == PF_BC_ZOUHE_SHEAR && (z == 0 || z == k.nz - 1)) || on_inout(k, n, z)) {
    float g[Q];
#pragma unroll
    for (int d = 0; d < Q; ++d) g[d] = q[d] * k.hs[wcls(d)];
    if (first) {
      ld_u<float>(ubuf, n, drho, ux, uy, uz);
    } else {
      float px = k.body_f[0], py = k.body_f[1], pz = k.body_f[2];
      if (fp) ld_force<float>(Fp, n, px, py, pz);
      node_state<float>(k, g, z, n, true, px, py, pz, drho, ux, uy, uz);
    }
    collide<float>(g, drho, ux, uy, uz, Fx, Fy, Fz, om, sf);
#pragma unroll
    for (int d = 0; d < Q; ++d) q[d] = g[d] * k.hinv[wcls(d)];
    return;
  }
  if (!fc && !fp && !first && k.nobody) {
    // interior node without any force (the quiet pass: most of the
    // lattice): the moments and the collision polynomial without their
    // force terms, which are exact zeros in the general form below
    const float s1 = k.hs[1], s2 = k.hs[2];
    const float ax = q[1] + q[2] + q[3] + q[4] + q[5] + q[6];
    const float dg = q[7] + q[8] + q[9] + q[10] + q[11] + q[12] + q[13] + q[14] + q[15] + q[16] + q[17] + q[18];
    const float drh = k.hs[0] * q[0] + s1 * ax + s2 * dg;
    const float jx = s1 * (q[1] - q[2]) + s2 * ((q[7] + q[8] + q[9] + q[10]) - (q[11] + q[12] + q[13] + q[14]));
    const float jy = s1 * (q[3] - q[4]) + s2 * ((q[7] + q[11] + q[15] + q[16]) - (q[8] + q[12] + q[17] + q[18]));
    const float jz = s1 * (q[5] - q[6]) + s2 * ((q[9] + q[13] + q[15] + q[17]) - (q[10] + q[14] + q[16] + q[18]));
    const float irho = __frcp_rn(1.0f + drh);
    const float vx = jx * irho, vy = jy * irho, vz = jz * irho;
    const float omr = om * (1.0f + drh), is = k.isig;
    const float A = (om * drh - 1.5f * omr * (vx * vx + vy * vy + vz * vz)) * is;
    const float B = 3.0f * omr * is, C = 4.5f * omr * is;
    const float omc = 1.0f - om;
    q[0] = omc * q[0] + A;
#pragma unroll
    for (int d = 1; d < Q; ++d) {
      if (opp(d) < d) continue;
      const int o = opp(d);
      const float cu = cdot<float>(d, vx, vy, vz);
      const float even = A + cu * (C * cu);
      const float odd = B * cu;
      q[d] = omc * q[d] + (even + odd);
      q[o] = omc * q[o] + (even - odd);
    }
    return;
  }
  if (first) {
    ld_u<float>(ubuf, n, drho, ux, uy, uz);
  } else {
    float px = k.body_f[0], py = k.body_f[1], pz = k.body_f[2];
    if (fp) ld_force<float>(Fp, n, px, py, pz);
    const float s1 = k.hs[1], s2 = k.hs[2];
    const float ax = q[1] + q[2] + q[3] + q[4] + q[5] + q[6];
    const float dg = q[7] + q[8] + q[9] + q[10] + q[11] + q[12] + q[13] + q[14] + q[15] + q[16] + q[17] + q[18];
    drho = k.hs[0] * q[0] + s1 * ax + s2 * dg;
    const float jx = s1 * (q[1] - q[2]) + s2 * ((q[7] + q[8] + q[9] + q[10]) - (q[11] + q[12] + q[13] + q[14]));
    const float jy = s1 * (q[3] - q[4]) + s2 * ((q[7] + q[11] + q[15] + q[16]) - (q[8] + q[12] + q[17] + q[18]));
    const float jz = s1 * (q[5] - q[6]) + s2 * ((q[9] + q[13] + q[15] + q[17]) - (q[10] + q[14] + q[16] + q[18]));
    // one correctly rounded reciprocal instead of three divisions: the
    // FP16 pass is bound by its instruction issue, and the difference (an
    // ulp of FP32) is far below the store's FP16 rounding
    const float hk = 0.5f * k.kmom_f, irho = __frcp_rn(1.0f + drho);
    ux = (jx + hk * px) * irho;
    uy = (jy + hk * py) * irho;
    uz = (jz + hk * pz) * irho;
  }
  const float rho = 1.0f + drho;
  const float usq = ux * ux + uy * uy + uz * uz;
  const float uF = ux * Fx + uy * Fy + uz * Fz;
  const float omr = om * rho, is = k.isig;
  const float A = (om * drho - 1.5f * omr * usq - 3.0f * sf * uF) * is;
  const float B = 3.0f * omr * is, C = 4.5f * omr * is, D = 3.0f * sf * is, E = 9.0f * sf * is;
  const float omc = 1.0f - om;
  q[0] = omc * q[0] + A;
#pragma unroll
  for (int d = 1; d < Q; ++d) {
    if (opp(d) < d) continue;
    const int o = opp(d);
    const float cu = cdot<float>(d, ux, uy, uz);
    const float cF = cdot<float>(d, Fx, Fy, Fz);
    const float even = A + cu * (C * cu + E * cF);
    const float odd = B * cu + D * cF;
    q[d] = omc * q[d] + (even + odd);
    q[o] = omc * q[o] + (even - odd);
  }
}

// One node of the direct-gather step: pull, moments with the previous
// force, collision with the current force, store; clears the previous force.
// FAST: no bounce-back face and 32-bit population indices (gather_fast).
template <class S, class R, bool FAST>
__device__ __forceinline__ void lbm_node(const LatticeConst& k, const S* __restrict__ gin, S* __restrict__ gout,
                                         const R4<R>* Fc, R4<R>* Fp, const R4<R>* ubuf, int x, int y, int z,
                                         unsigned fc, unsigned fp, int first) {
  const size_t N = (size_t)k.N;
  const size_t n = (size_t)x + (size_t)k.nx * ((size_t)y + (size_t)k.ny * z);
  if constexpr (std::is_same<S, __half>::value) {
    float q[Q];
    if constexpr (FAST) gather_fast<S, R, true>(k, gin, x, y, z, q);
    else gather<S, R, true>(k, gin, x, y, z, q);
    node_q(k, q, z, first, n, ubuf, Fp, fp, Fc, fc);
    S* p = gout + n;
#pragma unroll
    for (int d = 0; d < Q; ++d) {
      *p = __float2half_rn(q[d]);
      p += N;
    }
    if (fp) zero_force<R>(Fp, n);
    return;
  }
  R g[Q];
  if constexpr (FAST) gather_fast<S, R>(k, gin, x, y, z, g);
  else gather<S, R>(k, gin, x, y, z, g);
  R drho, ux, uy, uz;
  if (first) {
    // the first collision after an upload uses the uploaded density and
    // velocity, and its populations are the uploaded fIN (no boundary pass)
    ld_u<R>(ubuf, n, drho, ux, uy, uz);
  } else {
    R px = kv<R>(k.body[0], k.body_f[0]), py = kv<R>(k.body[1], k.body_f[1]), pz = kv<R>(k.body[2], k.body_f[2]);
    if (fp) ld_force<R>(Fp, n, px, py, pz);
    node_state<R>(k, g, z, n, true, px, py, pz, drho, ux, uy, uz);
  }
  collide_node<R>(k, g, drho, ux, uy, uz, Fc, n, fc, kv<R>(k.kcoll, k.kcoll_f), kv<R>(k.omega, k.omega_f));
  // one pointer stepped by N: a 64-bit add per store instead of forming
  // each direction's index (16 % fewer instructions in the FP32 pass)
  S* p = gout + n;
#pragma unroll
  for (int d = 0; d < Q; ++d) {
    st<S, R>(p, g[d], d, k);
    p += N;
  }
  if (fp) zero_force<R>(Fp, n);
}

// Zeroes the Morse cell counters (after this step's Morse pass, before the
// position update bins the elements again).
__device__ __forceinline__ void zero_bins(int* bin_count, int ncells, Control* ctl, size_t tid, size_t tot) {
  for (size_t c = tid; c < (size_t)ncells; c += tot) bin_count[c] = 0;
  if (tid == 0) ctl->occupied = 0;
}

// Direct-gather step over the lattice, one force brick (32 x-nodes of a row)
// per warp, four consecutive bricks per CTA.  mode:
//   kPassAll     every brick;
//   kPassUnflag  bricks not flagged for this step's force (the flagged ones
//                are left to lbm_list_k, after the spreading);
//   kPassNear    unflagged bricks of the near region (near[par] set);
//   kPassFar     the far region (near[par] clear) of step ctl->far_step,
//                which may run while the previous step's spreading,
//                flagged-brick pass and interpolation are still running: it
//                takes its parity and first-step flag from far_step /
//                far_first, and has no force (no far brick is flagged in
//                this step or the previous one).
//   kPassQuiet   bricks without force in the previous step (flags of the
//                previous step, known when the step starts), taken as
//                without force in this step too; bricks that gain a force in
//                this step are computed again by lbm_list_k, whose list holds
//                the bricks flagged in this step or the previous one.  So
//                this pass waits for no flagging; a marker moves far less
//                than a node per step, and the bricks computed twice are the
//                few a stencil enters in this step.
enum : int { kPassAll = 0, kPassUnflag = 1, kPassNear = 4, kPassFar = 3, kPassQuiet = 5 };
// bid / nblk: the CTA's index and the number of CTAs of this lattice's pass
// (the launch is one-dimensional over groups of four bricks in lattice order)
template <class S, class R, bool FAST>
__device__ __forceinline__ void lbm_step_body(const LatticeConst& k, S* gA, S* gB, R4<R>* FA, R4<R>* FB,
                                              R4<R>* ubuf, unsigned* flA, unsigned* flB, int* bin_count,
                                              int ncells, int mode, const unsigned char* nearA,
                                              const unsigned char* nearB, Control* ctl, int bid, int nblk) {
  const bool far = mode == kPassFar, quiet = mode == kPassQuiet;
  if (quiet ? ctl->qskip != 0 : ctl->done != 0) return;
  const int par = (int)((far ? ctl->far_step : (quiet ? ctl->qstep : ctl->step)) & 1);
  const S* __restrict__ gin = par ? gB : gA;
  S* __restrict__ gout = par ? gA : gB;
  const R4<R>* Fc = par ? FB : FA;
  R4<R>* Fp = par ? FA : FB;
  unsigned* flp = par ? flA : flB;
  const unsigned* flc = par ? flB : flA;
  // one brick (32 x-nodes of a row) per warp, bricks in lattice order: rows
  // narrower than a CTA leave no warp idle
  const int brick = bid * (kLbmBlock / kBrickX) + (int)(threadIdx.x >> 5);
  if (bin_count)
    zero_bins(bin_count, ncells, ctl, (size_t)bid * blockDim.x + threadIdx.x, (size_t)nblk * blockDim.x);
  if (brick >= k.nbricks) return;  // whole warp
  const int yz = brick / k.nbx;
  const int x = (brick - yz * k.nbx) * kBrickX + (int)(threadIdx.x & 31), y = yz % k.ny, z = yz / k.ny;
  // whole warp: one brick
  if (mode == kPassNear || far) {
    const unsigned char* nr = par ? nearB : nearA;
    const bool is_near = nr[brick] != 0;
    if (is_near == far) return;
  }
  if (far) {
    if (x < k.nx) lbm_node<S, R, FAST>(k, gin, gout, Fc, Fp, ubuf, x, y, z, 0u, 0u, ctl->far_first);
    return;
  }
  if (quiet) {
    if (flp[brick]) return;
    if (x < k.nx) lbm_node<S, R, FAST>(k, gin, gout, Fc, Fp, ubuf, x, y, z, 0u, 0u, ctl->qfirst);
    return;
  }
  const unsigned fc = flc[brick];
  if (mode != kPassAll && fc) return;
  const unsigned fp = flp[brick];
  if (x < k.nx) lbm_node<S, R, FAST>(k, gin, gout, Fc, Fp, ubuf, x, y, z, fc, fp, ctl->first);
  __syncwarp();
  if ((threadIdx.x & 31) == 0 && fp) flp[brick] = 0;
}
template <class S, class R, bool FAST>
__global__ void __launch_bounds__(kLbmBlock) lbm_step_k(LatticeConst k, S* gA, S* gB, R4<R>* FA, R4<R>* FB,
                                                        R4<R>* ubuf, unsigned* flA, unsigned* flB, int* bin_count,
                                                        int ncells, int mode, const unsigned char* nearA,
                                                        const unsigned char* nearB, Control* ctl) {
  lbm_step_body<S, R, FAST>(k, gA, gB, FA, FB, ubuf, flA, flB, bin_count, ncells, mode, nearA, nearB, ctl,
                            blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------- vector step
// The direct-gather step with V consecutive x-nodes per thread and every
// population plane moved as one aligned V-element vector per thread (8 or 16
// bytes): FP16 stores V = 4 or 8 halves, FP32 V = 2 or 4 floats.  For a
// direction with c_x = +1 (-1) the pull needs each node's left (right)
// neighbour in the same source row: the thread's own vector supplies all
// but one, the neighbouring lane's vector the last (a warp shuffle), and
// lanes whose neighbour segment lies in another warp, another row or an
// idle lane load that one element directly (periodic wrap at the row ends).
// Per node the arithmetic is lbm_node's, in the same order, so the results
// are bit-identical to the one-node-per-thread kernel (FP16: node_q on the
// stored q, two nodes per packed conversion); the populations are
// overwritten in place (a carry keeps each c_x = +1 input for the next
// node).  Lattices without bounce-back faces whose nx is a multiple of V.
template <class S, int V>
struct VecIO;
template <int V>
struct VecIO<float, V> {
  static constexpr int W = V;  // 32-bit words per vector
  __device__ static void load(const float* p, unsigned w[W]) {
    if constexpr (V == 4) {
      const uint4 a = __ldg(reinterpret_cast<const uint4*>(p));
      w[0] = a.x; w[1] = a.y; w[2] = a.z; w[3] = a.w;
    } else {
      const uint2 a = __ldg(reinterpret_cast<const uint2*>(p));
      w[0] = a.x; w[1] = a.y;
    }
  }
  __device__ static void store(float* p, const unsigned w[W]) {
    if constexpr (V == 4) *reinterpret_cast<uint4*>(p) = make_uint4(w[0], w[1], w[2], w[3]);
    else *reinterpret_cast<uint2*>(p) = make_uint2(w[0], w[1]);
  }
  __device__ static unsigned bits(const unsigned w[W], int i) { return w[i]; }
  __device__ static unsigned load_bits(const float* p) { return __float_as_uint(__ldg(p)); }
  __device__ static float value(unsigned b) { return __uint_as_float(b); }
  __device__ static void put(unsigned w[W], int i, float v) { w[i] = __float_as_uint(v); }
};
template <int V>
struct VecIO<__half, V> {
  static constexpr int W = V / 2;
  __device__ static void load(const __half* p, unsigned w[W]) {
    if constexpr (V == 8) {
      const uint4 a = __ldg(reinterpret_cast<const uint4*>(p));
      w[0] = a.x; w[1] = a.y; w[2] = a.z; w[3] = a.w;
    } else if constexpr (V == 4) {
      const uint2 a = __ldg(reinterpret_cast<const uint2*>(p));
      w[0] = a.x; w[1] = a.y;
    } else {
      w[0] = __ldg(reinterpret_cast<const unsigned*>(p));
    }
  }
  __device__ static void store(__half* p, const unsigned w[W]) {
    if constexpr (V == 8) *reinterpret_cast<uint4*>(p) = make_uint4(w[0], w[1], w[2], w[3]);
    else if constexpr (V == 4) *reinterpret_cast<uint2*>(p) = make_uint2(w[0], w[1]);
    else *reinterpret_cast<unsigned*>(p) = w[0];
  }
  __device__ static unsigned bits(const unsigned w[W], int i) { return (w[i >> 1] >> (16 * (i & 1))) & 0xffffu; }
  __device__ static unsigned load_bits(const __half* p) { return (unsigned)__half_as_ushort(__ldg(p)); }
};

// The pull of one V-node segment (row, sx) for every population plane:
// vector loads from the source rows, and for the x-shifted planes the one
// element outside the vector, from the lane holding the neighbouring segment
// of the same row (warp shuffle) or loaded directly.  Every lane of the warp
// calls it; lanes without `active` load nothing.
template <class S, int V>
__device__ __forceinline__ void vec_pull(const LatticeConst& k, const S* __restrict__ gin, bool active,
                                         unsigned row, unsigned sx, unsigned w[Q][VecIO<S, V>::W],
                                         unsigned edge[Q]) {
  using IO = VecIO<S, V>;
  const int lane = threadIdx.x & 31;
  const unsigned am = __ballot_sync(0xffffffffu, active);
  const unsigned nx = (unsigned)k.nx, ny = (unsigned)k.ny, nz = (unsigned)k.nz, N = (unsigned)k.N;
  const unsigned spr = nx / V, x0 = sx * V, y = row % ny, z = row / ny;
  // the source rows of the pull (periodic / Zou/He axes wrap)
  const unsigned ys[3] = {y == 0 ? ny - 1 : y - 1, y, y + 1 == ny ? 0u : y + 1};
  const unsigned zs[3] = {z == 0 ? nz - 1 : z - 1, z, z + 1 == nz ? 0u : z + 1};
  if (active) {
#pragma unroll
    for (int d = 0; d < Q; ++d) IO::load(gin + ((unsigned)d * N + nx * (ys[1 - cy(d)] + ny * zs[1 - cz(d)]) + x0), w[d]);
  }
  // the lane before (after) holds the segment to the left (right) when it
  // is active and on the same row
  const unsigned prow = __shfl_up_sync(0xffffffffu, row, 1), psx = __shfl_up_sync(0xffffffffu, sx, 1);
  const unsigned nrow = __shfl_down_sync(0xffffffffu, row, 1), nsx = __shfl_down_sync(0xffffffffu, sx, 1);
  const bool left_in_warp = lane > 0 && ((am >> (lane - 1)) & 1u) && prow == row && psx + 1 == sx;
  const bool right_in_warp = lane < 31 && ((am >> (lane + 1)) & 1u) && nrow == row && nsx == sx + 1;
  const unsigned xl = sx == 0 ? nx - 1 : x0 - 1, xr = sx + 1 == spr ? 0u : x0 + V;
#pragma unroll
  for (int d = 0; d < Q; ++d) {
    if (cx(d) == 0) continue;
    const unsigned mine = cx(d) == 1 ? IO::bits(w[d], V - 1) : IO::bits(w[d], 0);
    const unsigned nb = cx(d) == 1 ? __shfl_up_sync(0xffffffffu, mine, 1) : __shfl_down_sync(0xffffffffu, mine, 1);
    const bool ok = cx(d) == 1 ? left_in_warp : right_in_warp;
    edge[d] = nb;
    if (active && !ok)
      edge[d] = IO::load_bits(gin + ((unsigned)d * N + nx * (ys[1 - cy(d)] + ny * zs[1 - cz(d)]) +
                                     (cx(d) == 1 ? xl : xr)));
  }
}

// The stored bits of population d at node i of the segment, after the pull
// (c_x = +1: the left neighbour, c_x = -1: the right one).  `carry` keeps the
// c_x = +1 inputs of the previous node once a node's outputs overwrite w.
template <class S, int V>
__device__ __forceinline__ unsigned vec_in(const unsigned w[Q][VecIO<S, V>::W], const unsigned edge[Q],
                                           const unsigned carry[Q], int d, int i) {
  using IO = VecIO<S, V>;
  if (cx(d) == 0) return IO::bits(w[d], i);
  if (cx(d) == 1) return i == 0 ? edge[d] : carry[d];
  return i == V - 1 ? edge[d] : IO::bits(w[d], i + 1);
}

// Collide-and-store of a pulled segment (node n0 .. n0+V-1 at height z):
// lbm_node's arithmetic per node, outputs written back over w and stored as
// vectors; clears the previous force of the segment's nodes.
template <class S, int V>
__device__ __forceinline__ void vec_collide_store(const LatticeConst& k, S* __restrict__ gout, unsigned w[Q][VecIO<S, V>::W],
                                                  const unsigned edge[Q], unsigned n0, unsigned z, const float4* Fc,
                                                  float4* Fp, const float4* ubuf, unsigned fc, unsigned fp, int first) {
  using IO = VecIO<S, V>;
  const unsigned N = (unsigned)k.N;
  unsigned carry[Q];
  if constexpr (std::is_same<S, __half>::value) {
    // two nodes at a time: their outputs share a 32-bit word of each plane
    // and are packed by one conversion
#pragma unroll
    for (int i = 0; i < V; i += 2) {
      float qa[Q], qb[Q];
#pragma unroll
      for (int d = 0; d < Q; ++d) {
        const unsigned ba = vec_in<S, V>(w, edge, carry, d, i);
        unsigned bb;
        if (cx(d) == 1) {
          bb = IO::bits(w[d], i);
          carry[d] = IO::bits(w[d], i + 1);
        } else {
          bb = vec_in<S, V>(w, edge, carry, d, i + 1);
        }
        qa[d] = __half2float(__ushort_as_half((unsigned short)ba));
        qb[d] = __half2float(__ushort_as_half((unsigned short)bb));
      }
      node_q(k, qa, (int)z, first, n0 + i, ubuf, Fp, fp, Fc, fc);
      node_q(k, qb, (int)z, first, n0 + i + 1, ubuf, Fp, fp, Fc, fc);
#pragma unroll
      for (int d = 0; d < Q; ++d) {
        const __half2 h = __floats2half2_rn(qa[d], qb[d]);
        w[d][i >> 1] = *reinterpret_cast<const unsigned*>(&h);
      }
      if (fp) {
        zero_force<float>(Fp, n0 + i);
        zero_force<float>(Fp, n0 + i + 1);
      }
    }
  } else {
    const float kc = k.kcoll_f, om = k.omega_f;
#pragma unroll
    for (int i = 0; i < V; ++i) {
      const unsigned n = n0 + i;
      float g[Q];
#pragma unroll
      for (int d = 0; d < Q; ++d) {
        const unsigned b = vec_in<S, V>(w, edge, carry, d, i);
        if (cx(d) == 1) carry[d] = IO::bits(w[d], i);
        g[d] = IO::value(b);
      }
      float drho, ux, uy, uz;
      if (first) {
        ld_u<float>(ubuf, n, drho, ux, uy, uz);
      } else {
        float px = k.body_f[0], py = k.body_f[1], pz = k.body_f[2];
        if (fp) ld_force<float>(Fp, n, px, py, pz);
        node_state<float>(k, g, (int)z, (size_t)n, true, px, py, pz, drho, ux, uy, uz);
      }
      collide_node<float>(k, g, drho, ux, uy, uz, Fc, n, fc, kc, om);
#pragma unroll
      for (int d = 0; d < Q; ++d) IO::put(w[d], i, g[d]);
      if (fp) zero_force<float>(Fp, n);
    }
  }
#pragma unroll
  for (int d = 0; d < Q; ++d) IO::store(gout + ((unsigned)d * N + n0), w[d]);
}

// The step over the whole lattice (kPassAll) or the bricks without force
// (kPassUnflag): segment `seg` of the lattice in lattice order.
template <class S, int V>
__device__ __forceinline__ void lbm_vec_body(const LatticeConst& k, S* gA, S* gB, float4* FA, float4* FB,
                                             float4* ubuf, unsigned* flA, unsigned* flB, int* bin_count,
                                             int ncells, int mode, Control* ctl, long long seg, long long tid,
                                             long long tot) {
  using IO = VecIO<S, V>;
  const bool quiet = mode == kPassQuiet;
  if (quiet ? ctl->qskip != 0 : ctl->done != 0) return;
  const int par = (int)((quiet ? ctl->qstep : ctl->step) & 1);
  const S* __restrict__ gin = par ? gB : gA;
  S* __restrict__ gout = par ? gA : gB;
  const float4* Fc = par ? FB : FA;
  float4* Fp = par ? FA : FB;
  unsigned* flp = par ? flA : flB;
  const unsigned* flc = par ? flB : flA;
  if (bin_count) zero_bins(bin_count, ncells, ctl, (size_t)tid, (size_t)tot);
  const unsigned nx = (unsigned)k.nx;
  const unsigned spr = nx / V;  // segments per row
  const long long nseg = k.N / V;
  const bool valid = seg < nseg;
  const unsigned row = valid ? (unsigned)(seg / spr) : 0u;
  const unsigned sx = valid ? (unsigned)(seg - (long long)row * spr) : 0u;
  const unsigned x0 = sx * V;
  const int brick = (int)(x0 / kBrickX + (unsigned)k.nbx * row);
  const unsigned fc = (valid && !quiet) ? flc[brick] : 0u;
  const bool active = valid && (quiet ? flp[brick] == 0u : (mode == kPassAll || !fc));
  unsigned w[Q][IO::W], edge[Q];
  vec_pull<S, V>(k, gin, active, row, sx, w, edge);
  const unsigned am = __ballot_sync(0xffffffffu, active);
  if (!active) return;
  const unsigned fp = flp[brick];
  vec_collide_store<S, V>(k, gout, w, edge, nx * row + x0, row / (unsigned)k.ny, Fc, Fp, ubuf, fc, fp,
                          quiet ? ctl->qfirst : ctl->first);
  __syncwarp(am);
  if (fp && (x0 % kBrickX) == 0) flp[brick] = 0;
}

// CTAs per SM the vector kernel is compiled for: FP32 with two nodes per
// thread at 72 registers (7 CTAs, no spills), FP16 with four at 96 (5 CTAs,
// 80 bytes spilled).  The extra resident warps hide more of the pass's
// memory latency: 0.2002 -> 0.1968 ms (FP32) and 0.1690 -> 0.1667 ms (FP16)
// per coupled step of the 256x128x128 channel against the compiler's own
// 78 and 124 registers; 64 registers (8 CTAs) spill and were slower.
template <class S, int V>
constexpr int vec_min_ctas() {
  return (sizeof(S) == 4 && V == 2) ? 7 : ((sizeof(S) == 2 && V == 4) ? 5 : 1);
}

template <class S, int V>
__global__ void __launch_bounds__(kLbmBlock, vec_min_ctas<S, V>()) lbm_vec_k(LatticeConst k, S* gA, S* gB, float4* FA, float4* FB,
                                                       float4* ubuf, unsigned* flA, unsigned* flB, int* bin_count,
                                                       int ncells, int mode, Control* ctl) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  lbm_vec_body<S, V>(k, gA, gB, FA, FB, ubuf, flA, flB, bin_count, ncells, mode, ctl, t, t,
                     (long long)gridDim.x * blockDim.x);
}

// Near region of a step from a per-brick word array (non-zero: set): every
// brick within rx bricks in x and ry, rz rows in y, z of a set brick, all
// axes wrapped (a superset is always safe).  src_mark: from the occupancy
// bits into near[step parity] (before the first pipelined step, with the
// flags' own reach added); else from this step's flags into near[next
// parity].
__global__ void __launch_bounds__(256) near_bricks_k(LatticeConst k, const unsigned* flA, const unsigned* flB,
                                                     const unsigned* mark, unsigned char* nearA,
                                                     unsigned char* nearB, int src_mark, int rx, int ry, int rz,
                                                     const Control* ctl) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= k.nbricks) return;
  const int par = (int)(ctl->step & 1);
  const unsigned* src = src_mark ? mark + (size_t)par * k.nbricks : (par ? flB : flA);
  unsigned char* dst = (src_mark ? par : par ^ 1) ? nearB : nearA;
  const int bx = w % k.nbx, y = (w / k.nbx) % k.ny, z = w / (k.nbx * k.ny);
  unsigned acc = 0;
  for (int dz = -rz; dz <= rz && !acc; ++dz) {
    const int zz = wrapi(z + dz, k.nz);
    for (int dy = -ry; dy <= ry; ++dy) {
      const int yy = wrapi(y + dy, k.ny);
      const unsigned* row = src + (size_t)k.nbx * (yy + (size_t)k.ny * zz);
      for (int dx = -rx; dx <= rx; ++dx) acc |= row[wrapi(bx + dx, k.nbx)];
    }
  }
  dst[w] = acc != 0u;
}

// far_sync: the next far pass computes the current step (before the first
// pipelined step); far_close: after a far pass.
__global__ void far_counter_k(Control* ctl, int sync) {
  if (sync) {
    ctl->far_step = ctl->step;
    ctl->far_first = ctl->first;
  } else {
    ctl->far_step = ctl->far_step + 1;
    ctl->far_first = 0;
  }
}

// The flagged bricks of this step (list[par]), one warp per brick.
template <class S, class R, bool FAST>
__device__ __forceinline__ void lbm_list_body(const LatticeConst& k, S* gA, S* gB, R4<R>* FA, R4<R>* FB,
                                              R4<R>* ubuf, unsigned* flA, unsigned* flB, const int* lA,
                                              const int* lB, int* bin_count, int ncells, unsigned* mark,
                                              Control* ctl, int bid, int nblk) {
  // the quiet pass of the next step may run as soon as this pass is done
  // (it reads this step's output, written by now, and skips the bricks
  // flagged in this step)
  if (bid == 0 && threadIdx.x == 0) {
    ctl->qstep = ctl->step + 1;
    ctl->qfirst = 0;
    ctl->qskip = ctl->done;
  }
  if (ctl->done) return;
  const int par = (int)(ctl->step & 1);
  const S* __restrict__ gin = par ? gB : gA;
  S* __restrict__ gout = par ? gA : gB;
  const R4<R>* Fc = par ? FB : FA;
  R4<R>* Fp = par ? FA : FB;
  unsigned* flp = par ? flA : flB;
  const int* list = par ? lB : lA;
  // this step's occupancy bits, all inside flagged bricks: cleared here, the
  // last reader, for the position update two steps on
  unsigned* mk = mark + (size_t)par * k.nbricks;
  const int cnt = ctl->active_count[par];
  const int first = ctl->first;
  if (bin_count)
    zero_bins(bin_count, ncells, ctl, (size_t)bid * blockDim.x + threadIdx.x, (size_t)nblk * blockDim.x);
  const int warps = kLbmBlock / 32;
  const int lane = threadIdx.x & 31;
  for (int b = bid * warps + (threadIdx.x >> 5); b < cnt; b += nblk * warps) {
    const int brick = list[b];
    const int bx = brick % k.nbx;
    const int y = (brick / k.nbx) % k.ny;
    const int z = brick / (k.nbx * k.ny);
    const int x = bx * kBrickX + lane;
    const unsigned fp = flp[brick];
    if (x < k.nx) lbm_node<S, R, FAST>(k, gin, gout, Fc, Fp, ubuf, x, y, z, 1u, fp, first);
    __syncwarp();
    if (lane == 0) {
      if (fp) flp[brick] = 0;
      mk[brick] = 0u;
    }
  }
}
template <class S, class R, bool FAST>
__global__ void __launch_bounds__(kLbmBlock) lbm_list_k(LatticeConst k, S* gA, S* gB, R4<R>* FA, R4<R>* FB,
                                                        R4<R>* ubuf, unsigned* flA, unsigned* flB, const int* lA,
                                                        const int* lB, int* bin_count, int ncells, unsigned* mark,
                                                        Control* ctl) {
  lbm_list_body<S, R, FAST>(k, gA, gB, FA, FB, ubuf, flA, flB, lA, lB, bin_count, ncells, mark, ctl, blockIdx.x,
                            gridDim.x);
}

// ------------------------------------------------------------ row-staged step
// The same fused step with its loads staged through shared memory: a CTA of
// kRowThreads threads owns tiles of `rpt` consecutive x-rows (rpt * nx <= 256).
// For a tile and a direction d the source row (y - cy, z - cz) of plane d --
// or, through a bounce-back face in y or z, the tile's own row of plane
// opp(d) -- is one contiguous run of nx populations, copied by a bulk
// asynchronous copy that completes on the stage's "full" mbarrier.  Rows of
// directions with cx != 0 also get 16-byte halos (the periodic neighbours of
// the row's ends), so the pull's x shift is a constant offset into shared
// memory.  Row layout of a stage: [Q][DS] populations, row rr of direction d
// at d * DS + rr * (nx + 2H), H = 16 / sizeof(S) halo elements per side.
// Every warp owns one 32-node force brick of one row.  `stages` tiles are in
// flight per CTA: a warp arrives on the stage's "empty" barrier when done
// with it, warp 0 refills the stage once all warps have arrived.  The
// persistent grid walks the tiles in order.
constexpr int kRowThreads = 256;
constexpr int kMaxStages = 4;
constexpr unsigned kWaitSliceNs = 20000;                 // suspend hint of one try_wait
constexpr unsigned long long kWaitLimitNs = 1000000000ull;  // a stage is given up after 1 s

__constant__ int c_cx[Q] = {0, 1, -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0};
__constant__ int c_cy[Q] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1};
__constant__ int c_cz[Q] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1};
__constant__ int c_opp[Q] = {0, 2, 1, 4, 3, 6, 5, 12, 11, 14, 13, 8, 7, 10, 9, 18, 17, 16, 15};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect(uint64_t* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_try_wait_hint(uint64_t* b, unsigned parity, unsigned hint_ns) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity), "r"(hint_ns)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Wait for phase `parity` of a stage barrier: the waiting thread is
// suspended in the barrier (up to kWaitSliceNs per try) instead of spinning;
// false if the phase has not completed after limit_ns (0: one test without
// waiting, the test setting that makes the give-up path run).
__device__ __forceinline__ bool mbar_wait(uint64_t* b, unsigned parity, unsigned long long limit_ns) {
  if (mbar_try_wait(b, parity)) return true;
  if (limit_ns == 0) return false;
  const unsigned long long t0 = global_ns();
  for (;;) {
    if (mbar_try_wait_hint(b, parity, kWaitSliceNs)) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(b))
               : "memory");
}

// directions with cy == wy (wy != 0) or cz == wz (wz != 0), as a bit mask
__host__ __device__ constexpr unsigned dir_mask(int wy, int wz) {
  unsigned m = 0;
  for (int d = 0; d < Q; ++d)
    if ((wy != 0 && cy(d) == wy) || (wz != 0 && cz(d) == wz)) m |= 1u << d;
  return m;
}

template <class S, class R>
__device__ __forceinline__ R from_store(S v, int d, const LatticeConst& k);
template <>
__device__ __forceinline__ double from_store<double, double>(double v, int, const LatticeConst&) { return v; }
template <>
__device__ __forceinline__ float from_store<float, float>(float v, int, const LatticeConst&) { return v; }
template <>
__device__ __forceinline__ float from_store<__half, float>(__half v, int d, const LatticeConst& k) {
  return __half2float(v) * k.hs[wcls(d)];
}

template <class S, class R, int DS>
__global__ void __launch_bounds__(kRowThreads, sizeof(R) == 8 ? 1 : 3) lbm_rows_k(
    LatticeConst k, S* gA, S* gB, R4<R>* FA, R4<R>* FB, R4<R>* ubuf, unsigned* flA, unsigned* flB, int* bin_count,
    int ncells, int rpt, int stages, Control* ctl) {
  if (ctl->done) return;
  constexpr int kWarps = kRowThreads / 32;
  constexpr int H = 16 / (int)sizeof(S);  // halo elements per side
  extern __shared__ __align__(128) unsigned char s_raw[];
  __shared__ __align__(8) uint64_t s_full[kMaxStages], s_empty[kMaxStages];
  __shared__ int4 s_info[kMaxStages][kWarps];  // (y, z, own-row mask) of each staged row
  const long long step = ctl->step;
  const int par = (int)(step & 1);
  const S* __restrict__ gin = par ? gB : gA;
  S* __restrict__ gout = par ? gA : gB;
  R4<R>* Fc = par ? FB : FA;
  R4<R>* Fp = par ? FA : FB;
  unsigned* flp = par ? flA : flB;
  const unsigned* flc = par ? flB : flA;
  const int first = ctl->first;
  const int nx = k.nx, ny = k.ny, nz = k.nz;
  const int RS = nx + 2 * H;  // staged row length
  const int rows = ny * nz;
  const int ntiles = (rows + rpt - 1) / rpt;
  const size_t N = (size_t)k.N;
  const unsigned row_bytes = (unsigned)(nx * sizeof(S));
  S* sbuf = reinterpret_cast<S*>(s_raw);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool bbx = k.bc[0] == PF_BC_BOUNCEBACK, bby = k.bc[1] == PF_BC_BOUNCEBACK,
             bbz = k.bc[2] == PF_BC_BOUNCEBACK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < stages; ++s) {
      mbar_init(&s_full[s], 1);
      mbar_init(&s_empty[s], kWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  // Warp 0 stages local tile i (the CTA's i-th tile) into stage i % stages:
  // lanes < nr write the row descriptors, lane 0 arms the full barrier (its
  // release publishes the descriptors), the lanes then issue the copies, one
  // (direction, row) per lane: the row, and for cx != 0 its two halos.
  auto issue = [&](int i) {
    const int tile = blockIdx.x + i * gridDim.x;
    const int s = i % stages;
    const int r0 = tile * rpt;
    const int nr = min(rpt, rows - r0);
    if (lane < nr) {
      const int r = r0 + lane, y = r % ny, z = r / ny;
      unsigned mask = 0;
      if (bby && y == 0) mask |= dir_mask(1, 0);
      if (bby && y == ny - 1) mask |= dir_mask(-1, 0);
      if (bbz && z == 0) mask |= dir_mask(0, 1);
      if (bbz && z == nz - 1) mask |= dir_mask(0, -1);
      s_info[s][lane] = make_int4(y, z, (int)mask, 0);
    }
    __syncwarp();
    // 10 of the 19 directions have cx != 0: two 16-byte halos per row each
    if (lane == 0) mbar_arrive_expect(&s_full[s], (unsigned)nr * ((unsigned)Q * row_bytes + 10u * 32u));
    __syncwarp();
    S* st0 = sbuf + (size_t)s * Q * DS;
    for (int c = lane; c < Q * nr; c += 32) {
      const int d = c / nr, rr = c - d * nr;
      const int4 inf = s_info[s][rr];
      const S* src;
      if ((inf.z >> d) & 1) {
        src = gin + (size_t)c_opp[d] * N + (size_t)(r0 + rr) * nx;
      } else {
        int sy = inf.x - c_cy[d], sz = inf.y - c_cz[d];
        sy = sy < 0 ? sy + ny : (sy >= ny ? sy - ny : sy);
        sz = sz < 0 ? sz + nz : (sz >= nz ? sz - nz : sz);
        src = gin + (size_t)d * N + ((size_t)sy + (size_t)ny * sz) * nx;
      }
      S* dst = st0 + (size_t)d * DS + (size_t)rr * RS;
      bulk_load(dst + H, src, row_bytes, &s_full[s]);
      if (c_cx[d] != 0) {
        bulk_load(dst, src + (nx - H), 16u, &s_full[s]);
        bulk_load(dst + H + nx, src, 16u, &s_full[s]);
      }
    }
  };

  const R kc = kv<R>(k.kcoll, k.kcoll_f);
  const R om = kv<R>(k.omega, k.omega_f);
  // One node; p points at the node's column in direction 0 of its staged row.
  // Called by whole warps (a warp's 32 nodes are one force brick, whose
  // previous-force flag the warp clears).
  auto node = [&](const S* p, int x, int r, int4 inf, unsigned fc, unsigned fp) {
    const int z = inf.y;
    const unsigned mask = (unsigned)inf.z;
    const size_t n = (size_t)r * nx + x;
    R g[Q];
    if (mask == 0) {
      // interior row: every direction pulls from x - cx (halos cover the ends)
#pragma unroll
      for (int d = 0; d < Q; ++d) g[d] = from_store<S, R>(p[d * DS - cx(d)], d, k);
    } else {
      // row on a bounce-back face in y or z: own-row directions are unshifted
#pragma unroll
      for (int d = 0; d < Q; ++d) {
        const bool own = (cy(d) != 0 || cz(d) != 0) && ((mask >> d) & 1u);
        g[d] = from_store<S, R>(own ? p[d * DS] : p[d * DS - cx(d)], d, k);
      }
    }
    if (bbx && (x == 0 || x == nx - 1)) {
      // bounce-back x face: the node's own opp(d) population
#pragma unroll
      for (int d = 0; d < Q; ++d) {
        if (cx(d) == 0) continue;
        const bool own = (cy(d) != 0 || cz(d) != 0) && ((mask >> d) & 1u);
        if (!own && ((cx(d) == 1 && x == 0) || (cx(d) == -1 && x == nx - 1)))
          g[d] = ld<S, R>(gin + (size_t)opp(d) * N + n, opp(d), k);
      }
    }
    const int brick = (x >> 5) + k.nbx * r;
    R drho, ux, uy, uz;
    if (first) {
      ld_u<R>(ubuf, n, drho, ux, uy, uz);
    } else {
      R px = kv<R>(k.body[0], k.body_f[0]), py = kv<R>(k.body[1], k.body_f[1]), pz = kv<R>(k.body[2], k.body_f[2]);
      if (fp) ld_force<R>(Fp, n, px, py, pz);
      node_state<R>(k, g, z, n, true, px, py, pz, drho, ux, uy, uz);
    }
    collide_node<R>(k, g, drho, ux, uy, uz, Fc, n, fc, kc, om);
    S* o = gout + n;
#pragma unroll
    for (int d = 0; d < Q; ++d)
      st<S, R>(o + (size_t)d * N, g[d], d, k);
    if (fp) zero_force<R>(Fp, n);
    __syncwarp();
    if (lane == 0 && fp) flp[brick] = 0;
  };

  const int my_tiles = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  int issued = 0;
  if (warp == 0)
    for (; issued < stages && issued < my_tiles; ++issued) issue(issued);
  // This thread's node of every tile (rpt * nx <= kRowThreads: at most one):
  // row rr0 of the tile, column x0.  Its brick flags are loaded one tile
  // ahead, so their latency hides behind the previous tile's work.
  const int rr0 = (int)threadIdx.x / nx;
  const int x0 = (int)threadIdx.x - rr0 * nx;
  const bool has_node = rr0 < rpt;
  auto flags_of = [&](int i, unsigned& fc, unsigned& fp) {
    fc = fp = 0;
    if (!has_node || i >= my_tiles) return;
    const int r = (blockIdx.x + i * gridDim.x) * rpt + rr0;
    if (r >= rows) return;
    const int brick = (x0 >> 5) + k.nbx * r;
    fc = flc[brick];
    fp = flp[brick];
  };
  unsigned fc_next, fp_next;
  flags_of(0, fc_next, fp_next);
  bool failed = false;
  int i = 0;
  for (; i < my_tiles; ++i) {
    const int s = i % stages;
    const int r0 = (blockIdx.x + i * gridDim.x) * rpt;
    const int nr = min(rpt, rows - r0);
    const unsigned fc = fc_next, fp = fp_next;
    flags_of(i + 1, fc_next, fp_next);
    if (!mbar_wait(&s_full[s], (unsigned)((i / stages) & 1), k.wait_ns)) { failed = true; break; }
    if (has_node && rr0 < nr)
      node(sbuf + (size_t)s * Q * DS + H + rr0 * RS + x0, x0, r0 + rr0, s_info[s][rr0], fc, fp);
    __syncwarp();
    if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&s_empty[s])) : "memory");
    if (warp == 0 && issued < my_tiles) {
      // stage s is free once every warp has arrived on its empty barrier
      if (!mbar_wait(&s_empty[s], (unsigned)((i / stages) & 1), k.wait_ns)) { failed = true; break; }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(issued++);
    }
  }
  if (failed) {
    if (lane == 0) atomicOr(&ctl->err, ERR_WAIT_TIMEOUT);
    // let the copies this CTA issued land before it exits (tiles
    // i .. issued-1 are the latest users of their stages); always with the
    // full limit, whatever the stage waits were given
    if (warp == 0)
      for (int j = i; j < issued; ++j) mbar_wait(&s_full[j % stages], (unsigned)((j / stages) & 1), kWaitLimitNs);
    return;
  }
  if (bin_count) zero_bins(bin_count, ncells, ctl, (size_t)blockIdx.x * blockDim.x + threadIdx.x,
                          (size_t)gridDim.x * blockDim.x);
}

// (rho, u/C) of the nodes of the active bricks after this step's stream and
// boundary conditions, with this step's force: input of the IBM interpolation
// (the reference's velocity_density, LB_kernel.cu:1108-1199).
template <class S, class R, bool FAST>
__device__ __forceinline__ void moments_body(const LatticeConst& k, const S* gA, const S* gB, const R4<R>* FA,
                                             const R4<R>* FB, R4<R>* ubuf, const int* lA, const int* lB,
                                             const Control* ctl, int bid, int nblk) {
  if (ctl->done) return;
  const int par = (int)(ctl->step & 1);
  const S* gnew = par ? gA : gB;
  const R4<R>* Fc = par ? FB : FA;
  const int* list = par ? lB : lA;
  const int cnt = ctl->active_count[par];
  const int warps = kLbmBlock / 32;
  const int lane = threadIdx.x & 31;
  for (int b = bid * warps + (threadIdx.x >> 5); b < cnt; b += nblk * warps) {
    const int brick = list[b];
    const int bx = brick % k.nbx;
    const int y = (brick / k.nbx) % k.ny;
    const int z = brick / (k.nbx * k.ny);
    const int x = bx * kBrickX + lane;
    if (x >= k.nx) continue;
    const size_t n = (size_t)x + (size_t)k.nx * ((size_t)y + (size_t)k.ny * z);
    R g[Q];
    if constexpr (FAST) gather_fast<S, R>(k, gnew, x, y, z, g);
    else gather<S, R>(k, gnew, x, y, z, g);
    R Fx = kv<R>(k.body[0], k.body_f[0]), Fy = kv<R>(k.body[1], k.body_f[1]), Fz = kv<R>(k.body[2], k.body_f[2]);
    ld_force<R>(Fc, n, Fx, Fy, Fz);
    R drho, ux, uy, uz;
    node_state<R>(k, g, z, n, true, Fx, Fy, Fz, drho, ux, uy, uz);
    st_u<R>(ubuf, n, drho, ux, uy, uz);
  }
}
template <class S, class R, bool FAST>
__global__ void __launch_bounds__(kLbmBlock) moments_active_k(LatticeConst k, const S* gA, const S* gB,
                                                              const R4<R>* FA, const R4<R>* FB, R4<R>* ubuf,
                                                              const int* lA, const int* lB, const Control* ctl) {
  moments_body<S, R, FAST>(k, gA, gB, FA, FB, ubuf, lA, lB, ctl, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------- batch kernels
// lattice passes of a fused batch: the job's LatticeConst is copied to shared
// memory (no aliasing with the populations the pass writes)
template <class S, class R, bool FAST>
__global__ void __launch_bounds__(kLbmBlock) lbm_step_batch_k(const BatchDesc* descs, const int* start, int nj,
                                                              int rows) {
  __shared__ LatticeConst s_k;
  const int j = batch_job_of(start, nj, blockIdx.x);
  const BatchDesc& d = descs[j];
  cta_copy(s_k, d.L.k);
  __syncthreads();
  const Lattice& L = d.L;
  // `rows` groups of four bricks per CTA (amortizes the per-CTA set-up)
  const int segs = (s_k.nbricks + kLbmBlock / kBrickX - 1) / (kLbmBlock / kBrickX);
  for (int r = (blockIdx.x - start[j]) * rows, e = min(segs, r + rows); r < e; ++r)
    lbm_step_body<S, R, FAST>(s_k, (S*)L.g[0], (S*)L.g[1], (R4<R>*)L.F[0], (R4<R>*)L.F[1], (R4<R>*)L.ubuf,
                              L.flags[0], L.flags[1], nullptr, 0, kPassQuiet, L.near[0], L.near[1], d.ctl, r,
                              segs);
}
template <class S, class R, bool FAST>
__global__ void __launch_bounds__(kLbmBlock) lbm_list_batch_k(const BatchDesc* descs, const int* start, int nj) {
  __shared__ LatticeConst s_k;
  const int j = batch_job_of(start, nj, blockIdx.x);
  const BatchDesc& d = descs[j];
  cta_copy(s_k, d.L.k);
  __syncthreads();
  const Lattice& L = d.L;
  lbm_list_body<S, R, FAST>(s_k, (S*)L.g[0], (S*)L.g[1], (R4<R>*)L.F[0], (R4<R>*)L.F[1], (R4<R>*)L.ubuf,
                            L.flags[0], L.flags[1], L.list[0], L.list[1], nullptr, 0, L.mark, d.ctl,
                            blockIdx.x - start[j], start[j + 1] - start[j]);
}
template <class S, class R, bool FAST>
__global__ void __launch_bounds__(kLbmBlock) moments_batch_k(const BatchDesc* descs, const int* start, int nj) {
  __shared__ LatticeConst s_k;
  const int j = batch_job_of(start, nj, blockIdx.x);
  const BatchDesc& d = descs[j];
  cta_copy(s_k, d.L.k);
  __syncthreads();
  const Lattice& L = d.L;
  moments_body<S, R, FAST>(s_k, (const S*)L.g[0], (const S*)L.g[1], (const R4<R>*)L.F[0], (const R4<R>*)L.F[1],
                           (R4<R>*)L.ubuf, L.list[0], L.list[1], d.ctl, blockIdx.x - start[j],
                           start[j + 1] - start[j]);
}

// Full-lattice post-stream state in the reference's host layouts (double).
template <class S, class R>
__global__ void download_k(LatticeConst k, const S* gsrc, const R4<R>* Fsrc, const R4<R>* ubuf, int apply_bc,
                           int use_ubuf, double* fIN, double* fOUT, double* rho_o, double* u_o, double* F_o) {
  const size_t N = (size_t)k.N;
  const size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int x = (int)(n % k.nx), y = (int)((n / k.nx) % k.ny), z = (int)(n / ((size_t)k.nx * k.ny));
  R g[Q];
  gather<S, R>(k, gsrc, x, y, z, g);
  R Fx = kv<R>(k.body[0], k.body_f[0]), Fy = kv<R>(k.body[1], k.body_f[1]), Fz = kv<R>(k.body[2], k.body_f[2]);
  ld_force<R>(Fsrc, n, Fx, Fy, Fz);
  R drho, ux, uy, uz;
  if (use_ubuf) {
    ld_u<R>(ubuf, n, drho, ux, uy, uz);
  } else {
    node_state<R>(k, g, z, n, apply_bc != 0, Fx, Fy, Fz, drho, ux, uy, uz);
  }
  for (int d = 0; d < Q; ++d) {
    if (fIN) fIN[(size_t)d * N + n] = (double)g[d] + wgt(d);
    if (fOUT) fOUT[(size_t)d * N + n] = (double)ld<S, R>(gsrc + (size_t)d * N + n, d, k) + wgt(d);
  }
  if (rho_o) rho_o[n] = 1.0 + (double)drho;
  if (u_o) {
    u_o[n] = (double)ux * k.C;
    u_o[N + n] = (double)uy * k.C;
    u_o[2 * N + n] = (double)uz * k.C;
  }
  if (F_o) {
    F_o[n] = (double)Fx;
    F_o[N + n] = (double)Fy;
    F_o[2 * N + n] = (double)Fz;
  }
}

// Density and velocity (the units of download_k's u) at every stride-th
// node in x, y and z, as float planes [mz][my][mx] for the VTK dump.
template <class S, class R>
__global__ void fields_k(LatticeConst k, const S* gsrc, const R4<R>* Fsrc, const R4<R>* ubuf, int apply_bc,
                         int use_ubuf, int stride, int mx, int my, int mz, float* rho, float* ux, float* uy,
                         float* uz) {
  const size_t m = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= (size_t)mx * my * mz) return;
  const int x = (int)(m % mx) * stride, y = (int)((m / mx) % my) * stride, z = (int)(m / ((size_t)mx * my)) * stride;
  const size_t n = (size_t)x + (size_t)k.nx * ((size_t)y + (size_t)k.ny * z);
  R Fx = kv<R>(k.body[0], k.body_f[0]), Fy = kv<R>(k.body[1], k.body_f[1]), Fz = kv<R>(k.body[2], k.body_f[2]);
  ld_force<R>(Fsrc, n, Fx, Fy, Fz);
  R drho, vx, vy, vz;
  if (use_ubuf) {
    ld_u<R>(ubuf, n, drho, vx, vy, vz);
  } else {
    R g[Q];
    gather<S, R>(k, gsrc, x, y, z, g);
    node_state<R>(k, g, z, n, apply_bc != 0, Fx, Fy, Fz, drho, vx, vy, vz);
  }
  if (rho) rho[m] = (float)(1.0 + (double)drho);
  if (ux) {
    ux[m] = (float)((double)vx * k.C);
    uy[m] = (float)((double)vy * k.C);
    uz[m] = (float)((double)vz * k.C);
  }
}

// The device lattice of a new job in one pass over the nodes, every source
// word read once.  Node x takes its 19 initial populations f_d(x) -- the
// caller's fIN [19][N] (any address the device reads: device memory, pinned
// host memory, or pageable host memory where the GPU walks the host page
// tables), else the equilibrium of the initial flow -- and pushes each to
// the node that pulls it in the first step: g_d(x - c_d) = f_d(x) - w_d, so
// that the first pull reproduces fIN; where x + c_d lies beyond a
// bounce-back face, node x keeps g_d(x) = f_opp(d)(x) - w_d itself.  Every
// (node, direction) is written once.  (rho, u/C) for the first collision:
// the caller's rho_init / u_init, else the moments of f with the half-force
// shift and the Zou/He walls (fluid_initGPUKernel, semLB.cu:154-233), else
// the equilibrium's own.  The initial force loads into the step-before
// buffer and flags its bricks.  FP64 operations and their order are those of
// the host restatements (round-to-nearest intrinsics, no contraction), so
// FP64 jobs match them bit for bit.
template <class S, class R>
__global__ void lattice_init_k(LatticeConst k, InitSource src, S* g, R4<R>* Fprev, unsigned* flprev, R4<R>* ubuf) {
  const size_t N = (size_t)k.N;
  const size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int x = (int)(n % k.nx), y = (int)((n / k.nx) % k.ny), z = (int)(n / ((size_t)k.nx * k.ny));
  double f[Q];
  double r, u0, u1, u2;
  if (src.f) {
#pragma unroll
    for (int d = 0; d < Q; ++d) f[d] = src.f[(size_t)d * N + n];
    if (src.rho && src.u) {
      r = src.rho[n];
      u0 = src.u[n];
      u1 = src.u[N + n];
      u2 = src.u[2 * N + n];
    } else {
      double a = 0, b = 0, c = 0;
      r = 0;
      for (int d = 0; d < Q; ++d) {
        r = __dadd_rn(r, f[d]);
        a = __dadd_rn(a, __dmul_rn((double)cx(d), f[d]));
        b = __dadd_rn(b, __dmul_rn((double)cy(d), f[d]));
        c = __dadd_rn(c, __dmul_rn((double)cz(d), f[d]));
      }
      const double Fx = src.F ? src.F[n] : 0, Fy = src.F ? src.F[N + n] : 0, Fz = src.F ? src.F[2 * N + n] : 0;
      const double h = __dmul_rn(0.5, src.Fo);
      u0 = __ddiv_rn(__dadd_rn(__dmul_rn(a, src.C), __dmul_rn(__dmul_rn(h, Fx), src.dt)), r);
      u1 = __ddiv_rn(__dadd_rn(__dmul_rn(b, src.C), __dmul_rn(__dmul_rn(h, Fy), src.dt)), r);
      u2 = __ddiv_rn(__dadd_rn(__dmul_rn(c, src.C), __dmul_rn(__dmul_rn(h, Fz), src.dt)), r);
      if (src.zh && (z == 0 || z == k.nz - 1)) {
        u0 = 0;
        u2 = 0;
        u1 = z == 0 ? 0.0 : src.uw;
      }
    }
  } else {
    // equilibrium of rest, the caller's u_init / rho_init, or the Zou/He
    // channel's linear shear profile u_y = shear * z * dx / UMAX
    // (gpuSEM_LB.c:1206-1258)
    u0 = 0; u1 = 0; u2 = 0; r = 1.0;
    if (src.u) {
      u0 = src.u[n];
      u1 = src.u[N + n];
      u2 = src.u[2 * N + n];
    } else if (src.zh) {
      u1 = __ddiv_rn(__dmul_rn(__dmul_rn(src.shear, (double)z), src.dx), src.umax);
    }
    if (src.rho) r = src.rho[n];
    const double uu = __dadd_rn(__dadd_rn(__dmul_rn(u0, u0), __dmul_rn(u1, u1)), __dmul_rn(u2, u2));
    const double tail = __ddiv_rn(__dmul_rn(1.5, uu), src.C02);
#pragma unroll
    for (int d = 0; d < Q; ++d) {
      const double cu = __dmul_rn(3.0, __dadd_rn(__dadd_rn(__dmul_rn((double)cx(d), u0), __dmul_rn((double)cy(d), u1)),
                                                 __dmul_rn((double)cz(d), u2)));
      const double in = __dsub_rn(
          __dadd_rn(__dadd_rn(1.0, __ddiv_rn(cu, src.C0)), __ddiv_rn(__dmul_rn(__dmul_rn(0.5, cu), cu), src.C02)), tail);
      f[d] = __dmul_rn(__dmul_rn(r, wgt(d)), in);
    }
  }
#pragma unroll
  for (int d = 0; d < Q; ++d) {
    // push f_d(x) to x - c_d (periodic unless the face is bounce-back)
    int tx = x - cx(d), ty = y - cy(d), tz = z - cz(d);
    bool ok = true;
    if (tx < 0 || tx >= k.nx) { if (k.bc[0] == PF_BC_BOUNCEBACK) ok = false; else tx = (tx + k.nx) % k.nx; }
    if (ty < 0 || ty >= k.ny) { if (k.bc[1] == PF_BC_BOUNCEBACK) ok = false; else ty = (ty + k.ny) % k.ny; }
    if (tz < 0 || tz >= k.nz) { if (k.bc[2] == PF_BC_BOUNCEBACK) ok = false; else tz = (tz + k.nz) % k.nz; }
    if (ok)
      st<S, R>(g + (size_t)d * N + (size_t)tx + (size_t)k.nx * ((size_t)ty + (size_t)k.ny * tz), (R)(f[d] - wgt(d)),
               d, k);
    // x + c_d beyond a bounce-back face: node x keeps the reflected value
    const int sx = x + cx(d), sy = y + cy(d), sz = z + cz(d);
    const bool out = ((sx < 0 || sx >= k.nx) && k.bc[0] == PF_BC_BOUNCEBACK) ||
                     ((sy < 0 || sy >= k.ny) && k.bc[1] == PF_BC_BOUNCEBACK) ||
                     ((sz < 0 || sz >= k.nz) && k.bc[2] == PF_BC_BOUNCEBACK);
    if (out) st<S, R>(g + (size_t)d * N + n, (R)(f[opp(d)] - wgt(d)), d, k);
  }
  R fx = 0, fy = 0, fz = 0;
  if (src.F) { fx = (R)src.F[n]; fy = (R)src.F[N + n]; fz = (R)src.F[2 * N + n]; }
  if (fx != 0 || fy != 0 || fz != 0) {
    const int brick = x / kBrickX + k.nbx * (y + k.ny * z);
    flprev[brick] = 1u;
  }
  R4<R> v;
  v.x = fx; v.y = fy; v.z = fz; v.w = 0;
  Fprev[n] = v;
  st_u<R>(ubuf, n, (R)(r - 1.0), (R)(u0 / k.C), (R)(u1 / k.C), (R)(u2 / k.C));
}

template <class S, class R>
__global__ void conservation_k(LatticeConst k, const S* gsrc, double* out) {
  const size_t N = (size_t)k.N;
  const size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double m = 0, a = 0, b = 0, c = 0;
  if (n < N) {
    const int x = (int)(n % k.nx), y = (int)((n / k.nx) % k.ny), z = (int)(n / ((size_t)k.nx * k.ny));
    R g[Q];
    gather<S, R>(k, gsrc, x, y, z, g);
    if (k.bc[2] == PF_BC_ZOUHE_SHEAR && (z == 0 || z == k.nz - 1)) {
      if (z == 0) zouhe_bottom(g);
      else zouhe_top(g, kv<R>(k.uw, k.uw_f));
    }
    for (int d = 0; d < Q; ++d) {
      double f = (double)g[d] + wgt(d);
      m += f; a += cx(d) * f; b += cy(d) * f; c += cz(d) * f;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    m += __shfl_xor_sync(0xffffffffu, m, o);
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out, m); atomicAdd(out + 1, a); atomicAdd(out + 2, b); atomicAdd(out + 3, c);
  }
}

// Row-staged configuration: nx a multiple of 32 and at most 256 (each staged
// row is a multiple of 16 bytes, every warp owns one force brick, a tile of
// max(1, 256 / nx) rows with halos fits the direction stride DS of 272 or
// 384 populations); three stages when they fit beside two more CTAs on an
// SM, else two.
template <class S, class R, int DS>
bool rows_try(Lattice& L, int rpt) {
  const size_t stage = (size_t)Q * DS * sizeof(S);
  int stages = 3;
  if (3 * stage > 72 * 1024) stages = 2;
  const size_t smem = (size_t)stages * stage;
  if (cudaFuncSetAttribute(lbm_rows_k<S, R, DS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  int dev = 0, sms = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, lbm_rows_k<S, R, DS>, kRowThreads, smem) != cudaSuccess ||
      occ < 1) {
    cudaGetLastError();
    return false;
  }
  const int ntiles = (L.k.ny * L.k.nz + rpt - 1) / rpt;
  L.rows_rpt = rpt;
  L.rows_stages = stages;
  L.rows_smem = smem;
  L.rows_ds = DS;
  L.rows_grid = std::min(ntiles, sms * occ);
  return true;
}

// The direct-gather kernel is the default (it measured faster on the FP32
// 256x128x128 channel); PFGPU_LBM_KERNEL=rows selects the row-staged one.
template <class S, class R>
void rows_config(Lattice& L) {
  L.rows_stages = 0;
  const char* sel = getenv("PFGPU_LBM_KERNEL");
  if (!sel || strcmp(sel, "rows") != 0) return;
  const int nx = L.k.nx;
  if (nx % 32 != 0 || nx > kRowThreads) return;
  const int rpt = kRowThreads / nx;
  const int need = rpt * (nx + 2 * (16 / (int)sizeof(S)));
  if (need <= 272) rows_try<S, R, 272>(L, rpt);
  else if (need <= 384) rows_try<S, R, 384>(L, rpt);
}

// No bounce-back face and 19 N populations addressable with 32 bits.
inline bool fast_lattice(const Lattice& L) {
  return L.k.bc[0] != PF_BC_BOUNCEBACK && L.k.bc[1] != PF_BC_BOUNCEBACK && L.k.bc[2] != PF_BC_BOUNCEBACK &&
         19ull * (unsigned long long)L.k.N < (1ull << 32) && !getenv("PFGPU_GENERIC_GATHER");
}

// Nodes per thread of the vector step for this lattice, 0 for the
// one-node-per-thread kernel: FP32 2, FP16 4 (8-byte vectors; measured
// faster than 16-byte ones, whose registers halve the resident warps).  The
// vector step needs a lattice without bounce-back faces and nx a multiple
// of the width.  PFGPU_LBM_VEC=0 / 2 / 4 / 8 overrides (0: off).
template <class S>
int vec_width(const Lattice& L) {
  if (!fast_lattice(L)) return 0;
  int V = std::is_same<S, float>::value ? 2 : 4;
  if (const char* e = getenv("PFGPU_LBM_VEC")) {
    V = atoi(e);
    if (V == 8 && std::is_same<S, float>::value) V = 4;
  }
  if (V != 2 && V != 4 && V != 8) return 0;
  return (L.k.nx % V == 0) ? V : 0;
}

// part: 0 the whole lattice, 1 the bricks not flagged for this step's force,
// 2 the flagged bricks (after the spreading).
template <class S, class R>
cudaError_t step_impl(Lattice& L, Control* ctl, int part, int* bin_count, int ncells, cudaStream_t st) {
  if (L.rows_stages < 0) rows_config<S, R>(L);
  if (part == 0 && L.rows_stages > 0) {
    auto kern = L.rows_ds == 272 ? lbm_rows_k<S, R, 272> : lbm_rows_k<S, R, 384>;
    kern<<<L.rows_grid, kRowThreads, L.rows_smem, st>>>(L.k, (S*)L.g[0], (S*)L.g[1], (R4<R>*)L.F[0],
                                                       (R4<R>*)L.F[1], (R4<R>*)L.ubuf, L.flags[0], L.flags[1],
                                                       bin_count, ncells, L.rows_rpt, L.rows_stages, ctl);
    return cudaGetLastError();
  }
  if (part == 2) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int grid = sms * 8;
    const int need = (L.k.nbricks + kLbmBlock / 32 - 1) / (kLbmBlock / 32);
    if (grid > need) grid = need;
    auto kern = fast_lattice(L) ? lbm_list_k<S, R, true> : lbm_list_k<S, R, false>;
    kern<<<grid, kLbmBlock, 0, st>>>(L.k, (S*)L.g[0], (S*)L.g[1], (R4<R>*)L.F[0], (R4<R>*)L.F[1], (R4<R>*)L.ubuf,
                                     L.flags[0], L.flags[1], L.list[0], L.list[1], bin_count, ncells, L.mark,
                                     ctl);
    return cudaGetLastError();
  }
  if constexpr (!std::is_same<S, double>::value) {
    const int V = vec_width<S>(L);
    if (V > 0 && (part == 0 || part == 1 || part == kPassQuiet)) {
      const long long nseg = L.k.N / V;
      const unsigned vgrid = (unsigned)((nseg + kLbmBlock - 1) / kLbmBlock);
      void (*kern)(LatticeConst, S*, S*, float4*, float4*, float4*, unsigned*, unsigned*, int*, int, int, Control*);
      if constexpr (std::is_same<S, float>::value) kern = V == 4 ? lbm_vec_k<S, 4> : lbm_vec_k<S, 2>;
      else kern = V == 8 ? lbm_vec_k<S, 8> : (V == 4 ? lbm_vec_k<S, 4> : lbm_vec_k<S, 2>);
      kern<<<vgrid, kLbmBlock, 0, st>>>(L.k, (S*)L.g[0], (S*)L.g[1], (float4*)L.F[0], (float4*)L.F[1],
                                        (float4*)L.ubuf, L.flags[0], L.flags[1], bin_count, ncells, part, ctl);
      return cudaGetLastError();
    }
  }
  const unsigned grid = (unsigned)((L.k.nbricks + kLbmBlock / kBrickX - 1) / (kLbmBlock / kBrickX));
  auto kern = fast_lattice(L) ? lbm_step_k<S, R, true> : lbm_step_k<S, R, false>;
  kern<<<grid, kLbmBlock, 0, st>>>(L.k, (S*)L.g[0], (S*)L.g[1], (R4<R>*)L.F[0], (R4<R>*)L.F[1], (R4<R>*)L.ubuf,
                                   L.flags[0], L.flags[1], bin_count, ncells, part, L.near[0], L.near[1], ctl);
  return cudaGetLastError();
}
template <class S, class R>
cudaError_t moments_impl(Lattice& L, Control* ctl, cudaStream_t st) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int grid = sms * 8;
  const int need = (L.k.nbricks + kLbmBlock / 32 - 1) / (kLbmBlock / 32);
  if (grid > need) grid = need;
  auto kern = fast_lattice(L) ? moments_active_k<S, R, true> : moments_active_k<S, R, false>;
  kern<<<grid, kLbmBlock, 0, st>>>(L.k, (const S*)L.g[0], (const S*)L.g[1],
                                                    (const R4<R>*)L.F[0], (const R4<R>*)L.F[1], (R4<R>*)L.ubuf,
                                                    L.list[0], L.list[1], ctl);
  return cudaGetLastError();
}
template <class S, class R>
cudaError_t init_impl(Lattice& L, const InitSource& src, cudaStream_t st) {
  const size_t N = (size_t)L.k.N;
  lattice_init_k<S, R><<<(unsigned)((N + 255) / 256), 256, 0, st>>>(L.k, src, (S*)L.g[0], (R4<R>*)L.F[1],
                                                                     L.flags[1], (R4<R>*)L.ubuf);
  return cudaGetLastError();
}
template <class S, class R>
cudaError_t download_impl(Lattice& L, long long step, double* fIN, double* fOUT, double* rho, double* u, double* F,
                          cudaStream_t st) {
  const size_t N = (size_t)L.k.N;
  // latest post-collision buffer and force of the last step; before any
  // step: the uploaded state (no boundary pass yet, initial rho/u)
  const void* gsrc;
  const void* Fs;
  int apply_bc = 1, use_ubuf = 0;
  if (step == 0) {
    gsrc = L.g[0];
    Fs = L.F[1];
    apply_bc = 0;
    use_ubuf = 1;
  } else {
    const int last = (int)((step - 1) & 1);
    gsrc = last ? L.g[0] : L.g[1];
    Fs = L.F[last];
  }
  download_k<S, R><<<(unsigned)((N + 255) / 256), 256, 0, st>>>(L.k, (const S*)gsrc, (const R4<R>*)Fs,
                                                                (const R4<R>*)L.ubuf, apply_bc, use_ubuf, fIN,
                                                                fOUT, rho, u, F);
  return cudaGetLastError();
}
template <class S, class R>
cudaError_t fields_impl(Lattice& L, long long step, int stride, float* rho, float* ux, float* uy, float* uz,
                        cudaStream_t st) {
  const void* gsrc;
  const void* Fs;
  int apply_bc = 1, use_ubuf = 0;
  if (step == 0) {
    gsrc = L.g[0];
    Fs = L.F[1];
    apply_bc = 0;
    use_ubuf = 1;
  } else {
    const int last = (int)((step - 1) & 1);
    gsrc = last ? L.g[0] : L.g[1];
    Fs = L.F[last];
  }
  const int mx = (L.k.nx + stride - 1) / stride, my = (L.k.ny + stride - 1) / stride,
            mz = (L.k.nz + stride - 1) / stride;
  const size_t M = (size_t)mx * my * mz;
  fields_k<S, R><<<(unsigned)((M + 255) / 256), 256, 0, st>>>(L.k, (const S*)gsrc, (const R4<R>*)Fs,
                                                              (const R4<R>*)L.ubuf, apply_bc, use_ubuf, stride, mx,
                                                              my, mz, rho, ux, uy, uz);
  return cudaGetLastError();
}
template <class S, class R>
cudaError_t conservation_impl(Lattice& L, long long step, double* out, cudaStream_t st) {
  const size_t N = (size_t)L.k.N;
  const void* gsrc = step == 0 ? L.g[0] : (((step - 1) & 1) ? L.g[0] : L.g[1]);
  cudaMemsetAsync(out, 0, 4 * sizeof(double), st);
  conservation_k<S, R><<<(unsigned)((N + 255) / 256), 256, 0, st>>>(L.k, (const S*)gsrc, out);
  return cudaGetLastError();
}

}  // namespace

#define PF_DISPATCH(L, CALL)                              \
  switch ((L).precision) {                                \
    case PF_PREC_FP64: return CALL<double, double>;       \
    case PF_PREC_FP32: return CALL<float, float>;         \
    case PF_PREC_FP16: return CALL<__half, float>;        \
    default: return cudaErrorInvalidValue;                \
  }

cudaError_t lattice_init(Lattice& L, const InitSource& src, cudaStream_t st) {
  switch (L.precision) {
    case PF_PREC_FP64: return init_impl<double, double>(L, src, st);
    case PF_PREC_FP32: return init_impl<float, float>(L, src, st);
    case PF_PREC_FP16: return init_impl<__half, float>(L, src, st);
  }
  return cudaErrorInvalidValue;
}

cudaError_t lattice_step_part(Lattice& L, Control* ctl, int part, int* bin_count, int ncells, cudaStream_t st) {
  switch (L.precision) {
    case PF_PREC_FP64: return step_impl<double, double>(L, ctl, part, bin_count, ncells, st);
    case PF_PREC_FP32: return step_impl<float, float>(L, ctl, part, bin_count, ncells, st);
    case PF_PREC_FP16: return step_impl<__half, float>(L, ctl, part, bin_count, ncells, st);
  }
  return cudaErrorInvalidValue;
}
cudaError_t lattice_near(Lattice& L, Control* ctl, int from_mark, cudaStream_t st) {
  const int nb = L.k.nbricks;
  // from this step's flags: one brick in x, two rows in y and z (a marker's
  // base node moves at most one node per step, and a far node's pull must
  // not reach a flagged node); from the occupancy bits: plus the flags'
  // own reach (two nodes: one brick, two rows)
  const int rx = from_mark ? 2 : 1, ry = from_mark ? 4 : 2, rz = from_mark ? 4 : 2;
  near_bricks_k<<<(nb + 255) / 256, 256, 0, st>>>(L.k, L.flags[0], L.flags[1], L.mark, L.near[0], L.near[1],
                                                  from_mark, rx, ry, rz, ctl);
  return cudaGetLastError();
}
// the quiet pass of the current step, when no flagged-brick pass scheduled it
__global__ void quiet_prologue_k(Control* ctl) {
  ctl->qstep = ctl->step;
  ctl->qfirst = ctl->first;
  ctl->qskip = ctl->done;
}
cudaError_t lattice_quiet_prologue(Control* ctl, cudaStream_t st) {
  quiet_prologue_k<<<1, 1, 0, st>>>(ctl);
  return cudaGetLastError();
}
cudaError_t lattice_far_counter(Control* ctl, int sync, cudaStream_t st) {
  far_counter_k<<<1, 1, 0, st>>>(ctl, sync);
  return cudaGetLastError();
}
bool fast_gather(const Lattice& L) { return fast_lattice(L); }

template <class S, bool FAST>
static cudaError_t batch_lattice_impl(int kind, const BatchDesc* d, const int* start, int nj, int total, int rows,
                                      cudaStream_t st) {
  if (total <= 0) return cudaSuccess;
  switch (kind) {
    case BK_LBM_UNFLAGGED:
      lbm_step_batch_k<S, float, FAST><<<total, kLbmBlock, 0, st>>>(d, start, nj, rows);
      break;
    case BK_LBM_FLAGGED: lbm_list_batch_k<S, float, FAST><<<total, kLbmBlock, 0, st>>>(d, start, nj); break;
    case BK_MOMENTS: moments_batch_k<S, float, FAST><<<total, kLbmBlock, 0, st>>>(d, start, nj); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}
cudaError_t batch_launch_lattice(int kind, const BatchDesc* d, const int* start, int nj, int total, int precision,
                                 bool fast, int rows, cudaStream_t st) {
  if (precision == PF_PREC_FP32)
    return fast ? batch_lattice_impl<float, true>(kind, d, start, nj, total, rows, st)
                : batch_lattice_impl<float, false>(kind, d, start, nj, total, rows, st);
  if (precision == PF_PREC_FP16)
    return fast ? batch_lattice_impl<__half, true>(kind, d, start, nj, total, rows, st)
                : batch_lattice_impl<__half, false>(kind, d, start, nj, total, rows, st);
  return cudaErrorInvalidValue;
}

const char* lattice_pass_name(const Lattice& L) {
  if (L.rows_stages > 0) return "lbm_rows_k";
  int v = 0;
  if (L.precision == PF_PREC_FP32) v = vec_width<float>(L);
  else if (L.precision == PF_PREC_FP16) v = vec_width<__half>(L);
  return v ? "lbm_vec_k+lbm_list_k" : "lbm_step_k+lbm_list_k";
}

cudaError_t lattice_configure(Lattice& L) {
  switch (L.precision) {
    case PF_PREC_FP64: rows_config<double, double>(L); return cudaSuccess;
    case PF_PREC_FP32: rows_config<float, float>(L); return cudaSuccess;
    case PF_PREC_FP16: rows_config<__half, float>(L); return cudaSuccess;
  }
  return cudaErrorInvalidValue;
}
cudaError_t lattice_moments_active(Lattice& L, Control* ctl, cudaStream_t st) {
  switch (L.precision) {
    case PF_PREC_FP64: return moments_impl<double, double>(L, ctl, st);
    case PF_PREC_FP32: return moments_impl<float, float>(L, ctl, st);
    case PF_PREC_FP16: return moments_impl<__half, float>(L, ctl, st);
  }
  return cudaErrorInvalidValue;
}
cudaError_t lattice_download(Lattice& L, Control* ctl, long long step, double* fIN, double* fOUT, double* rho,
                             double* u, double* F, cudaStream_t st) {
  (void)ctl;
  switch (L.precision) {
    case PF_PREC_FP64: return download_impl<double, double>(L, step, fIN, fOUT, rho, u, F, st);
    case PF_PREC_FP32: return download_impl<float, float>(L, step, fIN, fOUT, rho, u, F, st);
    case PF_PREC_FP16: return download_impl<__half, float>(L, step, fIN, fOUT, rho, u, F, st);
  }
  return cudaErrorInvalidValue;
}
cudaError_t lattice_fields(Lattice& L, long long step, int stride, float* rho, float* ux, float* uy, float* uz,
                           cudaStream_t st) {
  switch (L.precision) {
    case PF_PREC_FP64: return fields_impl<double, double>(L, step, stride, rho, ux, uy, uz, st);
    case PF_PREC_FP32: return fields_impl<float, float>(L, step, stride, rho, ux, uy, uz, st);
    case PF_PREC_FP16: return fields_impl<__half, float>(L, step, stride, rho, ux, uy, uz, st);
  }
  return cudaErrorInvalidValue;
}
cudaError_t lattice_conservation(Lattice& L, long long step, double* out, cudaStream_t st) {
  switch (L.precision) {
    case PF_PREC_FP64: return conservation_impl<double, double>(L, step, out, st);
    case PF_PREC_FP32: return conservation_impl<float, float>(L, step, out, st);
    case PF_PREC_FP16: return conservation_impl<__half, float>(L, step, out, st);
  }
  return cudaErrorInvalidValue;
}

}  // namespace pf
