// pf_noalloc.cu -- the membrane force pass on caller-owned device arrays,
// without allocating: pfgpu_membrane_forces_noalloc.
//
// The pass needs per-call scratch (each node's triangle list, nodal and
// element normals, local strains, mean curvatures, one control word).  It
// lives in one file-scope device array of kNoAllocScratchBytes; the first
// call on a device looks up that array's address with cudaGetSymbolAddress
// (with the device current) and caches it per device.  No cudaMalloc,
// cudaFree or other allocating routine is called.
#include <algorithm>
#include <mutex>
#include <string>

#include "pf_internal.h"

namespace pf {
namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)PFGPU_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_addr_mu;
void* g_addr[kMaxDevices] = {};

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Checks the caller's topology on the device (the job path checks the same
// on the host before upload) and builds node -> its triangles in ascending
// order with the node's local index in each.  Thread q covers node q,
// triangle q and element q.  Any inconsistency -- a triangle index outside
// the nodes (or a corner outside the membrane), node_ntri outside 0..10 or
// unequal to the node's count in tri, a ring entry outside the membrane, a
// spring list outside the elements -- sets ERR_INPUT and done = 3, so the
// membrane kernels that follow on the stream return at once and read none
// of the bad indices.
__global__ void noalloc_topology_k(int T, int NN, int Em, int E, const int* tri, const int* node_ntri,
                                   const int* ring, const int* sp_ptr, const int* sp_nbr, int* node_tri,
                                   int* vert_local, Control* ctl) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  bool bad = false;
  if (q < T)
    for (int i = 0; i < 6; ++i) {
      const int v = tri[6 * q + i];
      if (v < 0 || v >= NN || (i < 3 && v >= Em)) bad = true;
    }
  if (q < NN) {
    int cnt = 0;
    for (int t = 0; t < T; ++t)
      for (int i = 0; i < 6; ++i)
        if (tri[6 * t + i] == q) {
          if (cnt < 10) {
            node_tri[10 * q + cnt] = t;
            if (q < Em) vert_local[10 * q + cnt] = i;
          }
          ++cnt;
        }
    for (int c = cnt; c < 10; ++c) {
      node_tri[10 * q + c] = -1;
      if (q < Em) vert_local[10 * q + c] = -1;
    }
    const int nt = node_ntri[q];
    if (cnt > 10 || nt != cnt) bad = true;
    if (q < Em && nt >= 0 && nt <= 10)
      for (int a = 0; a < nt; ++a) {
        const int r = ring[10 * q + a];
        if (r < 0 || r >= Em) bad = true;
      }
  }
  if (q < E) {
    const int b0 = sp_ptr[q], b1 = sp_ptr[q + 1];
    if ((q == 0 && b0 != 0) || b1 < b0) bad = true;
    else
      for (int s = b0; s < b1; ++s)
        if (sp_nbr[s] < 0 || sp_nbr[s] >= E) bad = true;
  }
  if (bad) {
    atomicOr(&ctl->err, ERR_INPUT);
    ctl->done = 3;
  }
}

}  // namespace
}  // namespace pf

using namespace pf;

extern "C" int pfgpu_membrane_forces_noalloc(const pf_membrane_args* a, void* stream) {
  if (!a) return report_error(PFGPU_ERR_INVALID, "membrane args are NULL");
  if (a->n_platelets < 1 || a->n_elem < 1 || a->n_membrane < 1 || a->n_membrane > a->n_elem || a->n_tri < 1 ||
      a->n_node < a->n_membrane)
    return report_error(PFGPU_ERR_INVALID, "membrane args: bad counts");
  if (a->precision < PF_PREC_FP64 || a->precision > PF_PREC_FP16)
    return report_error(PFGPU_ERR_INVALID, "membrane args: bad precision");
  if (a->membrane_forces & ~PF_MEM_ALL)
    return report_error(PFGPU_ERR_INVALID, "membrane args: only the PF_MEM_ALL terms (no FEM bending chain)");
  if (!a->X || !a->Y || !a->RY || !a->Z || !a->tri || !a->node_ntri || !a->ring || !a->spring_ptr || !a->S0 ||
      !a->S0_all || !a->V0 || !a->F_out)
    return report_error(PFGPU_ERR_INVALID, "membrane args: missing device array");
  const size_t P = (size_t)a->n_platelets, T = (size_t)a->n_tri, NN = (size_t)a->n_node, Em = (size_t)a->n_membrane;
  const size_t rb = a->precision == PF_PREC_FP64 ? 8 : 4;
  // scratch layout: control word, node triangle lists, then per platelet the
  // nodal normals, element normals, strains, curvatures
  const size_t off_ctl = 0;
  const size_t off_nt = align256(sizeof(Control));
  const size_t off_vl = off_nt + align256(NN * 10 * sizeof(int));
  const size_t off_nN = off_vl + align256(NN * 10 * sizeof(int));
  const size_t off_ne = off_nN + align256(P * NN * 3 * rb);
  const size_t off_S = off_ne + align256(P * T * 3 * rb);
  const size_t off_km = off_S + align256(P * T * rb);
  const size_t off_sv = off_km + align256(P * Em * rb);
  const size_t need = off_sv + align256(P * 2 * sizeof(double));
  if (need > kNoAllocScratchBytes) {
    const std::string msg = "membrane pass needs " + std::to_string(need) + " bytes of scratch; the static scratch holds " +
                            std::to_string(kNoAllocScratchBytes) + " (PFGPU_NOALLOC_SCRATCH_BYTES)";
    return report_error(PFGPU_ERR_INVALID, msg.c_str());
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return report_error(PFGPU_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return report_error(PFGPU_ERR_UNSUPPORTED, "device index out of range");
  unsigned char* base = nullptr;
  {
    // setup, once per device: the scratch array's device address
    std::lock_guard<std::mutex> lk(g_addr_mu);
    if (!g_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) return report_error(PFGPU_ERR_CUDA, cudaGetErrorString(e));
      g_addr[dev] = p;
    }
    base = static_cast<unsigned char*>(g_addr[dev]);
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  Control* ctl = reinterpret_cast<Control*>(base + off_ctl);
  int* node_tri = reinterpret_cast<int*>(base + off_nt);
  int* vert_local = reinterpret_cast<int*>(base + off_vl);
  // the control word must read zero (not done); every other scratch word is
  // written before it is read
  e = cudaMemsetAsync(ctl, 0, sizeof(Control), st);
  if (e != cudaSuccess) return report_error(PFGPU_ERR_CUDA, cudaGetErrorString(e));
  const size_t nthr = std::max(std::max(NN, T), (size_t)a->n_elem);
  noalloc_topology_k<<<(unsigned)((nthr + 127) / 128), 128, 0, st>>>(
      a->n_tri, a->n_node, a->n_membrane, a->n_elem, a->tri, a->node_ntri, a->ring, a->spring_ptr, a->spring_nbr,
      node_tri, vert_local, ctl);
  e = cudaGetLastError();
  if (e != cudaSuccess) return report_error(PFGPU_ERR_CUDA, cudaGetErrorString(e));
  PlateletConst k{};
  k.P = a->n_platelets; k.E = a->n_elem; k.Em = a->n_membrane; k.T = a->n_tri; k.NN = a->n_node;
  k.mask = a->membrane_forces;
  k.kspring = a->kspring; k.ks = a->ks; k.kv = a->kv; k.kbend = a->kbend; k.f0 = a->f0;
  const int prec = a->precision == PF_PREC_FP64 ? PF_PREC_FP64 : PF_PREC_FP32;
  e = membrane_forces_raw(k, prec, a->X, a->Y, a->RY, a->Z, a->tri, a->node_ntri, node_tri, vert_local, a->ring,
                          a->spring_ptr, a->spring_nbr, a->spring_L0, a->S0, a->S0_all, a->V0, base + off_nN,
                          base + off_ne, base + off_S, base + off_km,
                          a->S_V_out ? a->S_V_out : reinterpret_cast<double*>(base + off_sv), a->F_out, ctl, st);
  if (e != cudaSuccess) return report_error(PFGPU_ERR_CUDA, cudaGetErrorString(e));
  if (a->km_out) {
    e = cudaMemcpyAsync(a->km_out, base + off_km, P * Em * rb, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return report_error(PFGPU_ERR_CUDA, cudaGetErrorString(e));
  }
  return PFGPU_OK;
}

extern "C" size_t pfgpu_membrane_noalloc_scratch_bytes(void) { return kNoAllocScratchBytes; }

// Outcome of the last call on the current device: waits for `stream`, then
// copies the scratch's control word to the host (no allocation) and reports
// rejected inputs or a platelet too large for the pass.
extern "C" int pfgpu_membrane_noalloc_status(void* stream) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return report_error(PFGPU_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return report_error(PFGPU_ERR_UNSUPPORTED, "device index out of range");
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_addr_mu);
    base = g_addr[dev];
  }
  if (!base) return report_error(PFGPU_ERR_INVALID, "no membrane pass without allocation was made on this device");
  e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return report_error(PFGPU_ERR_CUDA, cudaGetErrorString(e));
  Control c;
  e = cudaMemcpy(&c, base, sizeof c, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return report_error(PFGPU_ERR_CUDA, cudaGetErrorString(e));
  if (c.err & ERR_INPUT)
    return report_error(PFGPU_ERR_INVALID,
                        "membrane pass without allocation: inconsistent topology (tri, node_ntri, ring or spring "
                        "arrays); F_out was not written");
  if (c.err & ERR_MEMBRANE_SIZE)
    return report_error(PFGPU_ERR_INVALID, "membrane pass without allocation: platelet too large for the pass");
  if (c.err) return report_error(PFGPU_ERR_CUDA, ("membrane pass error bits " + std::to_string(c.err)).c_str());
  return PFGPU_OK;
}
