// pf_input.cu -- the reference driver's host input: the parameter file
// (ParReader, gpuSEM_LB.c:148-343), the platelet surface mesh (NEUReader,
// gpuSEM_LB.c:345-404) and the membrane topology built from it
// (gpuSEM_LB.c:846-1055).  Host-only code; no CUDA call.
//
// Differences from the reference, by design: errors are returned (the
// reference prints and exits), index and count fields are range-checked,
// and the tables are CSR -- the mesh's bond lengths instead of the dense
// n_sce x n_sce bondLengths table, the node -> triangle lists and the
// ordered vertex rings instead of the [node][10] arrays (so no limit of ten
// triangles per node).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "pf_internal.h"

namespace {

int input_error(const std::string& msg) { return pf::report_error(PFGPU_ERR_INVALID, msg.c_str()); }

struct File {
  FILE* f = nullptr;
  explicit File(const char* path) : f(path ? fopen(path, "r") : nullptr) {}
  ~File() {
    if (f) fclose(f);
  }
};

}  // namespace

extern "C" {

// ParReader: "<KEYWORD> value" pairs in a fixed order; a keyword out of
// place fails with its name (the reference prints "Parameter Read Failed for
// <KEYWORD>" and exits).  host_param[3] (Kf0) is not in the file.
int pfgpu_read_parameter_file(const char* path, pf_parameter_file* out) {
  if (!path || !out) return input_error("pfgpu_read_parameter_file: NULL argument");
  File in(path);
  if (!in.f) return input_error(std::string("pfgpu_read_parameter_file: cannot open ") + path);
  pf_parameter_file p;
  memset(&p, 0, sizeof p);
  char key[64];
  auto keyword = [&](const char* want) {
    return fscanf(in.f, "%63s", key) == 1 && strcmp(key, want) == 0;
  };
  auto fail = [&](const char* want) {
    return input_error(std::string("pfgpu_read_parameter_file: expected ") + want);
  };
  struct Str {
    const char* key;
    char* dst;
  };
  const Str paths[3] = {{"PDB_PATH", p.pdb_path}, {"PSF_PATH", p.psf_path}, {"NEU_PATH", p.neu_path}};
  for (const Str& s : paths)
    if (!keyword(s.key) || fscanf(in.f, "%255s", s.dst) != 1) return fail(s.key);
  struct Flt {
    const char* key;
    float* dst;
  };
  const Flt head[3] = {{"DELTA_X", &p.dx}, {"DELTA_T", &p.dt}, {"SIM_TIME", &p.sim_time}};
  for (const Flt& s : head)
    if (!keyword(s.key) || fscanf(in.f, "%f", s.dst) != 1) return fail(s.key);
  struct Int {
    const char* key;
    int* dst;
  };
  const Int ints[4] = {{"OUT_FREQ", &p.out_freq}, {"MAX_CELL", &p.max_cell}, {"MAX_ELEM", &p.max_elem},
                       {"SURF_ELEM", &p.surf_elem}};
  for (const Int& s : ints)
    if (!keyword(s.key) || fscanf(in.f, "%d", s.dst) != 1) return fail(s.key);
  const Flt tail[6] = {{"RECEPTOR", &p.host_param[0]}, {"RANDOM_SEED", &p.host_param[1]},
                       {"K_SPRING", &p.host_param[2]}, {"Kr0", &p.host_param[4]},
                       {"SHEAR_RATE", &p.host_param[5]}, {"INIT_RHO", &p.host_param[6]}};
  for (const Flt& s : tail)
    if (!keyword(s.key) || fscanf(in.f, "%f", s.dst) != 1) return fail(s.key);
  *out = p;
  return PFGPU_OK;
}

// The two counts that open a NEU mesh file.
int pfgpu_neu_counts(const char* path, int* n_sce, int* n_tri) {
  if (!path || !n_sce || !n_tri) return input_error("pfgpu_neu_counts: NULL argument");
  File in(path);
  if (!in.f) return input_error(std::string("pfgpu_neu_counts: cannot open ") + path);
  if (fscanf(in.f, "%d %d", n_sce, n_tri) != 2 || *n_sce < 1 || *n_tri < 0)
    return input_error("pfgpu_neu_counts: bad header");
  return PFGPU_OK;
}

// NEUReader: n_sce records "index x y z" (1-based index, any order), then
// n_tri records "index a b n1 n2 n3" (1-based triangle and node indices; a,
// b unused).  Outputs the coordinates, tri3 [n_tri][3] (0-based) and the
// bond lengths of the triangle edges as CSR rows, ascending neighbour per
// element (bond_ptr [n_sce + 1], bond_nbr / bond_len [at most 6 n_tri]).
int pfgpu_read_neu(const char* path, double* X, double* Y, double* Z, int* tri3, int* bond_ptr, int* bond_nbr,
                   double* bond_len) {
  if (!path || !X || !Y || !Z || !tri3 || !bond_ptr || !bond_nbr || !bond_len)
    return input_error("pfgpu_read_neu: NULL argument");
  File in(path);
  if (!in.f) return input_error(std::string("pfgpu_read_neu: cannot open ") + path);
  int ns = 0, nt = 0;
  if (fscanf(in.f, "%d %d", &ns, &nt) != 2 || ns < 1 || nt < 0) return input_error("pfgpu_read_neu: bad header");
  for (int i = 0; i < ns; ++i) {
    int idx = 0;
    double x, y, z;
    if (fscanf(in.f, "%d %lf %lf %lf", &idx, &x, &y, &z) != 4) return input_error("pfgpu_read_neu: bad node record");
    if (idx < 1 || idx > ns) return input_error("pfgpu_read_neu: node index out of range");
    X[idx - 1] = x;
    Y[idx - 1] = y;
    Z[idx - 1] = z;
  }
  for (int i = 0; i < nt; ++i) {
    int idx = 0, a = 0, b = 0, n[3];
    if (fscanf(in.f, "%d %d %d %d %d %d", &idx, &a, &b, &n[0], &n[1], &n[2]) != 6)
      return input_error("pfgpu_read_neu: bad triangle record");
    if (idx < 1 || idx > nt) return input_error("pfgpu_read_neu: triangle index out of range");
    for (int k = 0; k < 3; ++k) {
      if (n[k] < 1 || n[k] > ns) return input_error("pfgpu_read_neu: triangle node out of range");
      tri3[3 * (idx - 1) + k] = n[k] - 1;
    }
  }
  // the edge lengths the reference writes into bondLengths[e1 + n_sce * e2]
  // (and its transpose) for each triangle edge, as sorted rows
  std::vector<std::map<int, double>> rows(ns);
  for (int t = 0; t < nt; ++t) {
    const int* v = tri3 + 3 * t;
    const int e[3][2] = {{v[0], v[1]}, {v[1], v[2]}, {v[2], v[0]}};
    for (const auto& ed : e) {
      const double dx = X[ed[0]] - X[ed[1]], dy = Y[ed[0]] - Y[ed[1]], dz = Z[ed[0]] - Z[ed[1]];
      const double dr = sqrt(dx * dx + dy * dy + dz * dz);
      rows[ed[0]][ed[1]] = dr;
      rows[ed[1]][ed[0]] = dr;
    }
  }
  int k = 0;
  bond_ptr[0] = 0;
  for (int i = 0; i < ns; ++i) {
    for (const auto& kv : rows[i]) {
      bond_nbr[k] = kv.first;
      bond_len[k] = kv.second;
      ++k;
    }
    bond_ptr[i + 1] = k;
  }
  return PFGPU_OK;
}

// Membrane topology (gpuSEM_LB.c:846-1055) of a closed triangle mesh.
//  tri6 [n_tri][6]: the three vertices, then a virtual node per shared edge
//    (numbered from n_vert in the order of the triangle pairs (i, j > i)
//    sharing it; the column is 3 + the sum of the edge's vertex slots, slot
//    sums 1..3; -1 where none);
//  node_ptr / node_tri: the triangles holding each node (vertices and
//    virtual nodes), for vertices reordered to follow the ring;
//  ring [node_ptr[n_vert]]: for vertex i, the ordered neighbour vertices,
//    ring[node_ptr[i] + j], j < node_ptr[i+1] - node_ptr[i];
//  normals [n_nodes][3]: minus the normalised mean of the unit normals
//    E12 x E13 of the node's triangles;
//  S0 [n_tri], *S0_all, *V0: rest areas, total area and the enclosed volume
//    (unit normal E13 x E12, centroid-weighted).
// Capacities: node_ptr n_vert + 3 n_tri + 1, node_tri 6 n_tri, ring 3 n_tri,
// normals 3 (n_vert + 3 n_tri).  *n_nodes receives the node count.
int pfgpu_build_topology(int n_vert, int n_tri, const int* tri3, const double* X, const double* Y, const double* Z,
                         int* tri6, int* n_nodes, int* node_ptr, int* node_tri, int* ring, double* normals,
                         double* S0, double* S0_all, double* V0) {
  if (n_vert < 1 || n_tri < 1 || !tri3 || !X || !Y || !Z || !tri6 || !n_nodes || !node_ptr || !node_tri || !ring ||
      !normals || !S0 || !S0_all || !V0)
    return input_error("pfgpu_build_topology: bad arguments");
  for (int i = 0; i < 3 * n_tri; ++i)
    if (tri3[i] < 0 || tri3[i] >= n_vert) return input_error("pfgpu_build_topology: vertex index out of range");
  const int T = n_tri;
  for (int i = 0; i < T; ++i)
    for (int k = 0; k < 6; ++k) tri6[6 * i + k] = k < 3 ? tri3[3 * i + k] : -1;
  // triangle pairs sharing an edge, visited in (i, j > i) order
  std::map<std::pair<int, int>, std::vector<int>> owners;
  for (int i = 0; i < T; ++i) {
    const int a = tri3[3 * i], b = tri3[3 * i + 1], c = tri3[3 * i + 2];
    const int e[3][2] = {{a, b}, {a, c}, {b, c}};
    for (const auto& ed : e) owners[{std::min(ed[0], ed[1]), std::max(ed[0], ed[1])}].push_back(i);
  }
  std::vector<std::vector<int>> later(T);
  for (const auto& kv : owners)
    if (kv.second.size() == 2) later[std::min(kv.second[0], kv.second[1])].push_back(std::max(kv.second[0], kv.second[1]));
  int newnode = n_vert;
  for (int i = 0; i < T; ++i) {
    std::sort(later[i].begin(), later[i].end());
    for (int j : later[i]) {
      int f1 = 0, f2 = 0, match = 0;
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l)
          if (tri6[6 * i + k] == tri6[6 * j + l]) {
            f1 += k;
            f2 += l;
            ++match;
          }
      if (match != 2) continue;
      if (f1 >= 1 && f1 <= 3) tri6[6 * i + 2 + f1] = newnode;
      if (f2 >= 1 && f2 <= 3) tri6[6 * j + 2 + f2] = newnode;
      ++newnode;
    }
  }
  if (T == 1) {
    newnode += 3;
    tri6[3] = 3;
    tri6[4] = 4;
    tri6[5] = 5;
  }
  // node -> triangles, in triangle order
  std::vector<std::vector<int>> share(newnode);
  for (int i = 0; i < T; ++i)
    for (int k = 0; k < 6; ++k) {
      const int nd = tri6[6 * i + k];
      if (nd == -1) break;
      share[nd].push_back(i);
    }
  // ring of each vertex: start from the vertex after i in its first
  // triangle, then walk to the triangle holding the current neighbour,
  // taking the vertex before it; the walked triangles move to the front
  std::vector<std::vector<int>> rings(n_vert);
  for (int i = 0; i < n_vert; ++i) {
    auto& sh = share[i];
    const int m = (int)sh.size();
    if (m == 0) continue;
    std::vector<int> r(m, -1);
    int node = -1;
    const int* t0 = tri6 + 6 * sh[0];
    for (int j = 0; j < 3; ++j)
      if (t0[j] == i) {
        node = j == 2 ? t0[0] : t0[j + 1];
        r[0] = node;
      }
    for (int j = 1; j < m; ++j)
      for (int k = j; k < m; ++k) {
        const int* t = tri6 + 6 * sh[k];
        bool hit = false;
        for (int l = 0; l < 3; ++l)
          if (t[l] == node) {
            hit = true;
            node = l == 0 ? t[2] : t[l - 1];
            r[j] = node;
            break;
          }
        if (hit) {
          std::swap(sh[j], sh[k]);
          break;
        }
      }
    rings[i] = r;
  }
  int k = 0;
  node_ptr[0] = 0;
  for (int nd = 0; nd < newnode; ++nd) {
    for (int t : share[nd]) node_tri[k++] = t;
    node_ptr[nd + 1] = k;
  }
  for (int i = 0; i < n_vert; ++i)
    for (size_t j = 0; j < rings[i].size(); ++j) ring[node_ptr[i] + (int)j] = rings[i][j];
  // reference normals
  for (int nd = 0; nd < newnode; ++nd) {
    double n[3] = {0, 0, 0};
    for (int t : share[nd]) {
      const int* v = tri6 + 6 * t;
      const double e12[3] = {X[v[1]] - X[v[0]], Y[v[1]] - Y[v[0]], Z[v[1]] - Z[v[0]]};
      const double e13[3] = {X[v[2]] - X[v[0]], Y[v[2]] - Y[v[0]], Z[v[2]] - Z[v[0]]};
      const double c[3] = {e12[1] * e13[2] - e12[2] * e13[1], e12[2] * e13[0] - e12[0] * e13[2],
                           e12[0] * e13[1] - e12[1] * e13[0]};
      const double nn = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
      for (int a = 0; a < 3; ++a) n[a] += c[a] / nn;
    }
    const int m = (int)share[nd].size();
    if (m) {
      for (double& v : n) v /= m;
      const double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      for (double& v : n) v /= -nn;
    }
    for (int a = 0; a < 3; ++a) normals[3 * nd + a] = n[a];
  }
  // rest areas and volume
  double area = 0, vol = 0;
  for (int i = 0; i < T; ++i) {
    const int* v = tri6 + 6 * i;
    const double P[3][3] = {{X[v[0]], Y[v[0]], Z[v[0]]}, {X[v[1]], Y[v[1]], Z[v[1]]}, {X[v[2]], Y[v[2]], Z[v[2]]}};
    double e12[3], e13[3], cc[3];
    for (int a = 0; a < 3; ++a) {
      e12[a] = P[1][a] - P[0][a];
      e13[a] = P[2][a] - P[0][a];
      cc[a] = 1 / 3.0 * (P[0][a] + P[1][a] + P[2][a]);
    }
    double n[3] = {e13[1] * e12[2] - e13[2] * e12[1], e13[2] * e12[0] - e13[0] * e12[2],
                   e13[0] * e12[1] - e13[1] * e12[0]};
    const double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (double& x : n) x /= nn;
    S0[i] = 0.5 * nn;
    area += S0[i];
    vol += 1 / 3.0 * (cc[0] * n[0] + cc[1] * n[1] + cc[2] * n[2]) * S0[i];
  }
  *S0_all = area;
  *V0 = vol;
  *n_nodes = newnode;
  return PFGPU_OK;
}

}  // extern "C"
