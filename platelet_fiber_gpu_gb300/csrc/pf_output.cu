// pf_output.cu -- the reference driver's element dumps (gpuSEM_LB.c:1327-1336
// opens them, :1376-1407 writes the initial frame, :1464-1494 one frame per
// output interval, :1533 the pause-time record), written from a job's state:
//   cellsPos.data    per element (cell by cell, elements in order): x, RY, z
//                    and z again ("for alignment in the octal dump"), one
//                    record per frame
//   cellsVel.data    the same four values of the velocity (vx, vy, vz, vz),
//   cellsForce.data  and of the force, initial frame only (the reference
//                    writes them once; its per-frame writes are commented out)
//   cells{Pos,Vel,Force}ASCII.dat  "Timestep ElemID X Y Z" tables, every frame
//   cellsPauseTime.dat            "<t * dt>, <seed>" appended at close
// Values are doubles as the reference writes them (PFGPU_OUT_FP64) or floats
// (PFGPU_OUT_FP32): four floats per element is the 16-byte record
// convBtoXYZ.py splits from `od -f` lines.  Host-only code.
#include <sys/stat.h>
#include <sys/types.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pf_internal.h"

extern "C" void pfgpu_job_elem_dims_(const pfgpu_job* j, int* P, int* E, double* dt);

struct pfgpu_output {
  pfgpu_job* job = nullptr;  // NULL: the caller hands the arrays to every frame
  long long step = 0;        // the last frame's step (arrays mode)
  int mode = PFGPU_OUT_FP64;
  int P = 0, E = 0;
  double dt = 0;
  FILE* f[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  std::vector<double> X, Y, RY, Z, V, F;
};

namespace {

enum { kPos, kVel, kForce, kPosA, kVelA, kForceA, kPause };
const char* kNames[7] = {"cellsPos.data",      "cellsVel.data",      "cellsForce.data",   "cellsPosASCII.dat",
                         "cellsVelASCII.dat", "cellsForceASCII.dat", "cellsPauseTime.dat"};

void close_all(pfgpu_output* o) {
  for (FILE*& fp : o->f)
    if (fp) {
      fclose(fp);
      fp = nullptr;
    }
}

int fetch(pfgpu_output* o) {
  return pfgpu_job_get_elements(o->job, o->X.data(), o->Y.data(), o->RY.data(), o->Z.data(), o->V.data(),
                                o->F.data());
}

// one binary record: a, b, c, c (doubles or floats)
bool put4(const pfgpu_output* o, FILE* fp, double a, double b, double c) {
  if (o->mode == PFGPU_OUT_FP32) {
    const float v[4] = {(float)a, (float)b, (float)c, (float)c};
    return fwrite(v, sizeof v, 1, fp) == 1;
  }
  const double v[4] = {a, b, c, c};
  return fwrite(v, sizeof v, 1, fp) == 1;
}

}  // namespace

namespace {
int open_files(pfgpu_output* o, const char* dir) {
  for (int i = 0; i < 7; ++i) {
    const std::string path = std::string(dir) + "/" + kNames[i];
    o->f[i] = fopen(path.c_str(), i == kPause ? "a+" : "wb+");
    if (!o->f[i]) {
      close_all(o);
      return pf::report_error(PFGPU_ERR_INVALID, ("pfgpu_output_open: cannot open " + path).c_str());
    }
  }
  return PFGPU_OK;
}
// initial frame (gpuSEM_LB.c:1376-1407): all three binaries, timestep 0
bool write_initial(pfgpu_output* o) {
  const size_t PE = (size_t)o->P * o->E;
  for (int i = kPosA; i <= kForceA; ++i) fprintf(o->f[i], "Timestep       ElemID        X         Y         Z\n");
  bool ok = true;
  for (int p = 0; p < o->P; ++p)
    for (int e = 0; e < o->E; ++e) {
      const size_t g = (size_t)p * o->E + e;
      ok = ok && put4(o, o->f[kPos], o->X[g], o->RY[g], o->Z[g]);
      fprintf(o->f[kPosA], "0      %d    %e   %e   %e\n ", e, o->X[g], o->RY[g], o->Z[g]);
      ok = ok && put4(o, o->f[kVel], o->V[g], o->V[PE + g], o->V[2 * PE + g]);
      fprintf(o->f[kVelA], "0      %d    %e   %e   %e\n ", e, o->V[g], o->V[PE + g], o->V[2 * PE + g]);
      ok = ok && put4(o, o->f[kForce], o->F[g], o->F[PE + g], o->F[2 * PE + g]);
      fprintf(o->f[kForceA], "0      %d    %e   %e   %e\n ", e, o->F[g], o->F[PE + g], o->F[2 * PE + g]);
    }
  return ok;
}
// gpuSEM_LB.c:1464-1494: positions to the binary dump, all three tables
bool write_frame(pfgpu_output* o, long long t) {
  const size_t PE = (size_t)o->P * o->E;
  bool ok = true;
  for (int p = 0; p < o->P; ++p)
    for (int e = 0; e < o->E; ++e) {
      const size_t g = (size_t)p * o->E + e;
      ok = ok && put4(o, o->f[kPos], o->X[g], o->RY[g], o->Z[g]);
      fprintf(o->f[kPosA], "%lld      %d  %e  %e  %e\n ", t, e, o->X[g], o->RY[g], o->Z[g]);
      fprintf(o->f[kVelA], "%lld      %d  %e  %e  %e\n ", t, e, o->V[g], o->V[PE + g], o->V[2 * PE + g]);
      fprintf(o->f[kForceA], "%lld      %d  %e  %e  %e\n ", t, e, o->F[g], o->F[PE + g], o->F[2 * PE + g]);
    }
  for (int i = 0; i < 6; ++i) fflush(o->f[i]);
  return ok;
}
void take(pfgpu_output* o, const double* X, const double* RY, const double* Z, const double* V, const double* F) {
  const size_t PE = (size_t)o->P * o->E;
  o->X.assign(X, X + PE);
  o->RY.assign(RY, RY + PE);
  o->Z.assign(Z, Z + PE);
  o->V.assign(V, V + 3 * PE);
  o->F.assign(F, F + 3 * PE);
}
}  // namespace

extern "C" {

int pfgpu_output_open(pfgpu_job* job, const char* dir, int mode, pfgpu_output** out) {
  if (!job || !dir || !out || (mode != PFGPU_OUT_FP64 && mode != PFGPU_OUT_FP32))
    return pf::report_error(PFGPU_ERR_INVALID, "pfgpu_output_open: bad arguments");
  *out = nullptr;
  pfgpu_output* o = new pfgpu_output;
  o->job = job;
  o->mode = mode;
  pfgpu_job_elem_dims_(job, &o->P, &o->E, &o->dt);
  const size_t PE = (size_t)o->P * o->E;
  o->X.resize(PE); o->Y.resize(PE); o->RY.resize(PE); o->Z.resize(PE);
  o->V.resize(3 * PE); o->F.resize(3 * PE);
  int rc = open_files(o, dir);
  if (rc == PFGPU_OK) rc = fetch(o);
  if (rc == PFGPU_OK && !write_initial(o)) rc = pf::report_error(PFGPU_ERR_INVALID, "pfgpu_output_open: write failed");
  if (rc) {
    close_all(o);
    delete o;
    return rc;
  }
  *out = o;
  return PFGPU_OK;
}

int pfgpu_output_open_arrays(const char* dir, int mode, int P, int E, double dt, const double* X, const double* RY,
                             const double* Z, const double* V, const double* F, pfgpu_output** out) {
  if (!dir || !out || (mode != PFGPU_OUT_FP64 && mode != PFGPU_OUT_FP32) || P < 0 || E < 0 || !X || !RY || !Z ||
      !V || !F)
    return pf::report_error(PFGPU_ERR_INVALID, "pfgpu_output_open_arrays: bad arguments");
  *out = nullptr;
  pfgpu_output* o = new pfgpu_output;
  o->mode = mode;
  o->P = P;
  o->E = E;
  o->dt = dt;
  take(o, X, RY, Z, V, F);
  int rc = open_files(o, dir);
  if (rc == PFGPU_OK && !write_initial(o))
    rc = pf::report_error(PFGPU_ERR_INVALID, "pfgpu_output_open_arrays: write failed");
  if (rc) {
    close_all(o);
    delete o;
    return rc;
  }
  *out = o;
  return PFGPU_OK;
}

int pfgpu_output_frame(pfgpu_output* o) {
  if (!o || !o->job) return pf::report_error(PFGPU_ERR_INVALID, "pfgpu_output_frame: NULL or arrays-mode handle");
  int rc = fetch(o);
  if (rc) return rc;
  const long long t = (long long)pfgpu_job_step_count(o->job);
  return write_frame(o, t) ? PFGPU_OK : pf::report_error(PFGPU_ERR_INVALID, "pfgpu_output_frame: write failed");
}

int pfgpu_output_frame_arrays(pfgpu_output* o, long long step, const double* X, const double* RY, const double* Z,
                              const double* V, const double* F) {
  if (!o || o->job || !X || !RY || !Z || !V || !F)
    return pf::report_error(PFGPU_ERR_INVALID, "pfgpu_output_frame_arrays: bad arguments");
  take(o, X, RY, Z, V, F);
  o->step = step;
  return write_frame(o, step) ? PFGPU_OK
                              : pf::report_error(PFGPU_ERR_INVALID, "pfgpu_output_frame_arrays: write failed");
}

int pfgpu_output_close(pfgpu_output* o, int seed) {
  if (!o) return PFGPU_OK;
  const long long t = o->job ? (long long)pfgpu_job_step_count(o->job) : o->step;
  // totalT * dt in the reference: int times float, in float
  fprintf(o->f[kPause], "%e, %d\n", (double)((float)t * (float)o->dt), seed);
  close_all(o);
  delete o;
  return PFGPU_OK;
}

}  // extern "C"

// writeVTK of the reference driver (gpuSEM_LB.c:1631-1709): the same file
// name pattern, XML header and value layout; Spacing carries the stride of
// downsampled fields.
extern "C" int pfgpu_write_vti(int t, int nx, int ny, int nz, int spacing, const float* rho, int write_rho,
                               const float* ux, const float* uy, const float* uz, int write_vel,
                               const char* directory, const char* filename) {
  if (nx < 1 || ny < 1 || nz < 1 || spacing < 1 || !directory || !filename || (write_rho && !rho) ||
      (write_vel && (!ux || !uy || !uz)))
    return pf::report_error(PFGPU_ERR_INVALID, "pfgpu_write_vti: bad arguments");
  mkdir(directory, 0777);
  char name[4096];
  snprintf(name, sizeof name, "%s/%s_%07d.vti", directory, filename, t);
  FILE* f = fopen(name, "w");
  if (!f) return pf::report_error(PFGPU_ERR_INVALID, "pfgpu_write_vti: cannot open the .vti file");
  fprintf(f, "<?xml version=\"1.0\"?>\n");
  fprintf(f, "<!-- gpuLBMflow ND ACMS -->\n");
  fprintf(f, "<VTKFile type=\"ImageData\" version=\"0.1\" byte_order=\"LittleEndian\">\n");
  fprintf(f, "  <ImageData WholeExtent=\"0 %d 0 %d 0 %d\" Origin=\"0 0 0\" Spacing=\"%d %d %d\">\n", nx - 1,
          ny - 1, nz - 1, spacing, spacing, spacing);
  fprintf(f, "  <Piece Extent=\"0 %d 0 %d 0 %d\">\n", nx - 1, ny - 1, nz - 1);
  fprintf(f, "    <PointData Scalars=\"scalars\">\n");
  const size_t row = (size_t)nx;
  if (write_rho) {
    fprintf(f, "      <DataArray type=\"Float32\" Name=\"Density\" NumberOfComponents=\"1\" format=\"ascii\">\n");
    for (size_t r = 0; r < (size_t)ny * nz; ++r) {
      for (size_t x = 0; x < row; ++x) fprintf(f, "%.4e ", rho[r * row + x]);
      fprintf(f, "\n");
    }
    fprintf(f, "      </DataArray>\n");
  }
  if (write_vel) {
    fprintf(f, "      <DataArray type=\"Float32\" Name=\"Velocity\" NumberOfComponents=\"3\" format=\"ascii\">\n");
    for (size_t r = 0; r < (size_t)ny * nz; ++r) {
      for (size_t x = 0; x < row; ++x) {
        const size_t i = r * row + x;
        fprintf(f, "%.4e %.4e %.4e ", ux[i], uy[i], uz[i]);
      }
      fprintf(f, "\n");
    }
    fprintf(f, "      </DataArray>\n");
  }
  fprintf(f, "    </PointData>\n");
  fprintf(f, "    <CellData>\n");
  fprintf(f, "    </CellData>\n");
  fprintf(f, "  </Piece>\n");
  fprintf(f, "  </ImageData>\n");
  fprintf(f, "</VTKFile>\n");
  const bool ok = !ferror(f);
  if (fclose(f) != 0 || !ok) return pf::report_error(PFGPU_ERR_INVALID, "pfgpu_write_vti: write failed");
  return PFGPU_OK;
}
