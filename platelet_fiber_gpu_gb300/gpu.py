"""ctypes binding of libpfgpu.so (the CUDA library).

There is no CPU fallback: if the library is missing or no CUDA device is
present, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from .scene import Scene

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libpfgpu.so"

PFGPU_OK, PFGPU_DONE = 0, 6
_STATUS = {1: "INVALID", 2: "CUDA", 3: "NOMEM", 4: "UNSUPPORTED", 5: "DEVICE", 6: "DONE"}

_lib = None


class PfgpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"pfgpu error {_STATUS.get(code, code)}: {msg}")
        self.code = code


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is not built; run platelet_fiber_gpu_gb300.build.build()")
        # independent jobs run on their own streams; more hardware work queues
        # than the default 8 keep them from serialising (read when the CUDA
        # context is created, so it only applies if nothing created it yet)
        os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
        L = C.CDLL(str(LIB_PATH))
        vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
        L.pfgpu_job_create.argtypes = [vp, C.c_int, C.c_double, C.POINTER(vp)]
        L.pfgpu_job_step.argtypes = [vp, C.c_int]
        L.pfgpu_job_step_graph.argtypes = [vp, C.c_int]
        L.pfgpu_job_sync.argtypes = [vp]
        L.pfgpu_job_get_lattice.argtypes = [vp, dp, dp, dp, dp, dp]
        L.pfgpu_job_get_elements.argtypes = [vp, dp, dp, dp, dp, dp, dp]
        L.pfgpu_job_get_bonds.argtypes = [vp, ip, ip, ip]
        L.pfgpu_job_get_fibrin.argtypes = [vp, dp, dp, dp, dp, dp]
        L.pfgpu_job_get_membrane.argtypes = [vp, dp, dp]
        L.pfgpu_job_conservation.argtypes = [vp, dp]
        L.pfgpu_job_step_count.restype = C.c_int64
        L.pfgpu_job_step_count.argtypes = [vp]
        L.pfgpu_job_device_bytes.restype = C.c_size_t
        L.pfgpu_job_device_bytes.argtypes = [vp]
        L.pfgpu_job_launches_per_step.argtypes = [vp]
        L.pfgpu_job_destroy.argtypes = [vp]
        L.pfgpu_job_lbm_kernel.restype = C.c_char_p
        L.pfgpu_job_lbm_kernel.argtypes = [vp]
        L.pfgpu_output_open.argtypes = [vp, C.c_char_p, C.c_int, C.POINTER(vp)]
        dpp = C.POINTER(C.c_double)
        L.pfgpu_read_parameter_file.argtypes = [C.c_char_p, vp]
        L.pfgpu_neu_counts.argtypes = [C.c_char_p, ip, ip]
        L.pfgpu_read_neu.argtypes = [C.c_char_p, dpp, dpp, dpp, ip, ip, ip, dpp]
        L.pfgpu_build_topology.argtypes = [C.c_int, C.c_int, ip, dpp, dpp, dpp, ip, ip, ip, ip, ip, dpp, dpp, dpp,
                                           dpp]
        fp = C.POINTER(C.c_float)
        L.pfgpu_job_get_fields.argtypes = [vp, C.c_int, fp, fp, fp, fp, ip]
        L.pfgpu_write_vti.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, fp, C.c_int, fp, fp, fp, C.c_int,
                                      C.c_char_p, C.c_char_p]
        L.pfgpu_output_frame.argtypes = [vp]
        L.pfgpu_output_close.argtypes = [vp, C.c_int]
        L.pfgpu_job_profile.argtypes = [vp, C.c_int, dp]
        L.pfgpu_job_get_cells.argtypes = [vp, ip, ip, ip, ip]
        L.pfgpu_profile_phase_count.restype = C.c_int
        L.pfgpu_profile_phase_name.restype = C.c_char_p
        L.pfgpu_profile_phase_name.argtypes = [C.c_int]
        L.pfgpu_scene_device_bytes.restype = C.c_size_t
        L.pfgpu_scene_device_bytes.argtypes = [vp, C.c_int]
        L.pfgpu_last_error.restype = C.c_char_p
        L.pfgpu_receptor_uniforms.argtypes = [C.c_uint64, C.c_int64, C.c_int64, dp]
        L.pfgpu_batch_create.argtypes = [C.c_size_t, C.POINTER(vp)]
        L.pfgpu_batch_admit.argtypes = [vp, vp, C.c_int, C.c_double, ip]
        L.pfgpu_batch_step.argtypes = [vp, C.c_int]
        L.pfgpu_batch_status.argtypes = [vp, C.c_int]
        L.pfgpu_batch_retire.argtypes = [vp, C.c_int]
        L.pfgpu_batch_job.restype = vp
        L.pfgpu_batch_job.argtypes = [vp, C.c_int]
        L.pfgpu_batch_bytes_in_use.restype = C.c_size_t
        L.pfgpu_batch_bytes_in_use.argtypes = [vp]
        L.pfgpu_batch_num_jobs.argtypes = [vp]
        L.pfgpu_batch_shape.argtypes = [vp, ip, ip]
        L.pfgpu_batch_set_stop.argtypes = [vp, C.c_int, C.c_int64]
        L.pfgpu_job_set_stop.argtypes = [vp, C.c_int64]
        L.pfgpu_batch_set_shape.argtypes = [vp, C.c_int, C.c_int, C.c_int]
        L.pfgpu_batch_destroy.argtypes = [vp]
        L.pfgpu_job_state_bytes.restype = C.c_size_t
        L.pfgpu_job_state_bytes.argtypes = [vp]
        L.pfgpu_job_save.argtypes = [vp, vp, C.c_size_t]
        L.pfgpu_job_restore.argtypes = [vp, vp, C.c_size_t]
        L.pfgpu_host_alloc.restype = vp
        L.pfgpu_host_alloc.argtypes = [C.c_size_t]
        L.pfgpu_host_free.argtypes = [vp]
        L.pfgpu_detach_uniform.restype = C.c_double
        L.pfgpu_detach_uniform.argtypes = [C.c_uint64, C.c_int64]
        _lib = L
    return _lib


class _PinnedOwner:
    def __init__(self, ptr):
        self.ptr = ptr

    def __del__(self):
        try:
            lib().pfgpu_host_free(self.ptr)
        except Exception:
            pass


def pinned(shape, dtype=np.float64) -> np.ndarray:
    """A numpy array in pinned, device-mapped host memory
    (pfgpu_host_alloc), freed when the last view of it goes."""
    dtype = np.dtype(dtype)
    n = int(np.prod(shape)) * dtype.itemsize
    ptr = lib().pfgpu_host_alloc(max(n, 1))
    if not ptr:
        raise PfgpuError(3, lib().pfgpu_last_error().decode(errors="replace"))
    buf = (C.c_byte * max(n, 1)).from_address(ptr)
    buf._owner = _PinnedOwner(ptr)
    return np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)


def _p(a, t=C.c_double):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def check(code: int, allow_done: bool = False) -> int:
    if code == PFGPU_OK or (allow_done and code == PFGPU_DONE):
        return code
    raise PfgpuError(code, lib().pfgpu_last_error().decode(errors="replace"))


def scene_device_bytes(scene: Scene, precision: int) -> int:
    c = scene.to_c()
    return lib().pfgpu_scene_device_bytes(C.byref(c), precision)


class Job:
    """A device-resident coupled simulation (pfgpu_job)."""

    def __init__(self, scene: Scene, precision: int = 1, fp16_scale: float = 0.0):
        self.scene = scene
        self.precision = precision
        self._c = scene.to_c()
        h = C.c_void_p()
        check(lib().pfgpu_job_create(C.byref(self._c), precision, fp16_scale, C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().pfgpu_job_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n: int = 1, graph: bool = True) -> int:
        f = lib().pfgpu_job_step_graph if graph else lib().pfgpu_job_step
        return check(f(self.h, int(n)), allow_done=True)

    def save(self) -> np.ndarray:
        """Snapshot of the job's whole device state (pfgpu_job_save)."""
        n = int(lib().pfgpu_job_state_bytes(self.h))
        buf = np.empty(n, dtype=np.uint8)
        check(lib().pfgpu_job_save(self.h, buf.ctypes.data_as(C.c_void_p), n))
        return buf

    def restore(self, snapshot: np.ndarray):
        """Loads a snapshot of a job of the same scene sizes and precision."""
        snap = np.ascontiguousarray(snapshot, dtype=np.uint8)
        check(lib().pfgpu_job_restore(self.h, snap.ctypes.data_as(C.c_void_p), snap.nbytes))

    def set_stop(self, stop_step: int):
        """The job stops by itself after step stop_step (0: never): later
        steps do nothing and step() returns PFGPU_DONE."""
        check(lib().pfgpu_job_set_stop(self.h, int(stop_step)))

    def profile(self, n: int) -> dict:
        """Per-phase device time (ms, summed over n serialised steps)."""
        k = lib().pfgpu_profile_phase_count()
        out = np.zeros(k)
        check(lib().pfgpu_job_profile(self.h, int(n), _p(out)), allow_done=True)
        return {lib().pfgpu_profile_phase_name(i).decode(): float(out[i]) for i in range(k)}

    @property
    def steps(self) -> int:
        return int(lib().pfgpu_job_step_count(self.h))

    @property
    def device_bytes(self) -> int:
        return int(lib().pfgpu_job_device_bytes(self.h))

    @property
    def launches_per_step(self) -> int:
        return int(lib().pfgpu_job_launches_per_step(self.h))

    @property
    def lbm_kernel(self) -> str:
        return lib().pfgpu_job_lbm_kernel(self.h).decode()

    def output(self, directory: str, fp32: bool = False) -> "Output":
        """The reference driver's element dumps in `directory` (initial frame
        written now); fp32: float records for convBtoXYZ.py."""
        return Output(self, directory, fp32)

    def lattice(self, fIN=True, fOUT=False, out=None):
        """fIN, fOUT [19, N], rho [N], u [3, N], F [3, N] (FP64); `out`: the
        caller's own arrays under those keys (C-contiguous float64, e.g.
        pinned()), written in place and returned."""
        N = self.scene.n_nodes
        if out is not None:
            for k, v in out.items():
                if v is not None and (v.dtype != np.float64 or not v.flags.c_contiguous):
                    raise ValueError(f"out[{k!r}] must be C-contiguous float64")
            a, b = out.get("fIN"), out.get("fOUT")
            rho, u, F = out.get("rho"), out.get("u"), out.get("F")
        else:
            a = np.zeros((19, N)) if fIN else None
            b = np.zeros((19, N)) if fOUT else None
            rho, u, F = np.zeros(N), np.zeros((3, N)), np.zeros((3, N))
        check(lib().pfgpu_job_get_lattice(self.h, _p(a), _p(b), _p(rho), _p(u), _p(F)))
        return dict(fIN=a, fOUT=b, rho=rho, u=u, F=F)

    def fields(self, stride: int = 1):
        """Density and velocity at every stride-th node, computed on the
        device: float32 arrays rho [mz, my, mx] and u [3, mz, my, mx]."""
        dims = (C.c_int * 3)()
        check(lib().pfgpu_job_get_fields(self.h, stride, None, None, None, None, dims))
        mx, my, mz = dims
        rho = np.zeros((mz, my, mx), dtype=np.float32)
        u = np.zeros((3, mz, my, mx), dtype=np.float32)
        check(lib().pfgpu_job_get_fields(self.h, stride, _p(rho, C.c_float), _p(u[0], C.c_float),
                                         _p(u[1], C.c_float), _p(u[2], C.c_float), dims))
        return dict(rho=rho, u=u)

    def write_vti(self, t: int, directory, filename: str = "LBMflow", stride: int = 1, write_rho: bool = True,
                  write_vel: bool = True):
        """The reference driver's VTK dump of this job's fields (downsampled
        by `stride` on the device)."""
        f = self.fields(stride)
        write_vti(t, f["rho"], f["u"], directory, filename, spacing=stride, write_rho=write_rho,
                  write_vel=write_vel)

    def elements(self, out=None):
        """X, Y, RY, Z [PE], V, F [3, PE]; `out`: the caller's arrays."""
        PE = self.scene.n_platelets * self.scene.n_elem
        if out is not None:
            X, Y, RY, Z, V, F = (out[k] for k in ("X", "Y", "RY", "Z", "V", "F"))
        else:
            X, Y, RY, Z = (np.zeros(PE) for _ in range(4))
            V, F = np.zeros((3, PE)), np.zeros((3, PE))
        check(lib().pfgpu_job_get_elements(self.h, _p(X), _p(Y), _p(RY), _p(Z), _p(V), _p(F)))
        return dict(X=X, Y=Y, RY=RY, Z=Z, V=V, F=F)

    def bonds(self):
        sc = self.scene
        st = np.zeros((sc.n_platelets, sc.n_rec, 3), dtype=np.int32)
        vwf = np.zeros((4, sc.ny, sc.nx), dtype=np.int32)
        tot = C.c_int(0)
        check(lib().pfgpu_job_get_bonds(self.h, _p(st, C.c_int), _p(vwf, C.c_int), C.byref(tot)))
        return dict(rec_state=st, vwf=vwf, total=tot.value)

    def fibrin(self):
        M = self.scene.n_fib
        X, Y, Z = np.zeros(M), np.zeros(M), np.zeros(M)
        V, F = np.zeros((3, M)), np.zeros((3, M))
        check(lib().pfgpu_job_get_fibrin(self.h, _p(X), _p(Y), _p(Z), _p(V), _p(F)))
        return dict(X=X, Y=Y, Z=Z, V=V, F=F)

    def membrane(self):
        sc = self.scene
        SV = np.zeros((sc.n_platelets, 2))
        km = np.zeros((sc.n_platelets, sc.n_membrane))
        check(lib().pfgpu_job_get_membrane(self.h, _p(SV), _p(km)))
        return dict(S_V=SV, km=km)

    def cells(self):
        """(cell of each element, count per cell, members per cell in id order, grid dims)"""
        sc = self.scene
        PE = sc.n_platelets * sc.n_elem
        nc = np.zeros(3, dtype=np.int32)
        cell_of = np.zeros(PE, dtype=np.int32)
        members = np.zeros(PE, dtype=np.int32)
        rc = max(sc.morse_intra[3], sc.morse_inter[3])
        dims = [max(1, int(np.floor(n * np.float64(np.float32(sc.dx)) / rc))) for n in (sc.nx, sc.ny, sc.nz)]
        counts = np.zeros(int(np.prod(dims)), dtype=np.int32)
        check(lib().pfgpu_job_get_cells(self.h, _p(cell_of, C.c_int), _p(counts, C.c_int), _p(members, C.c_int),
                                        _p(nc, C.c_int)))
        return cell_of, counts, members, nc

    def conservation(self):
        out = np.zeros(4)
        check(lib().pfgpu_job_conservation(self.h, _p(out)))
        return out


class Output:
    """cellsPos/Vel/Force.data, the ASCII tables and cellsPauseTime.dat of a
    job (pfgpu_output_*)."""

    def __init__(self, job: Job, directory: str, fp32: bool = False):
        self.job = job
        self.h = C.c_void_p()
        check(lib().pfgpu_output_open(job.h, str(directory).encode(), 1 if fp32 else 0, C.byref(self.h)))

    def frame(self):
        check(lib().pfgpu_output_frame(self.h))

    def close(self, seed: int = 0):
        if self.h:
            check(lib().pfgpu_output_close(self.h, int(seed)))
            self.h = C.c_void_p()


class _BatchJob(Job):
    """A job owned by a Batch (read-only view: the batch destroys it)."""

    def __init__(self, scene: Scene, handle):
        self.scene = scene
        self.h = C.c_void_p(handle)

    def close(self):
        self.h = None


def write_vti(t: int, rho, u, directory, filename: str = "LBMflow", spacing: int = 1, write_rho: bool = True,
              write_vel: bool = True):
    """pfgpu_write_vti: rho [nz, ny, nx] and u [3, nz, ny, nx] float32 host
    arrays to <directory>/<filename>_<t:07d>.vti (host-only)."""
    rho = np.ascontiguousarray(rho, dtype=np.float32)
    u = np.ascontiguousarray(u, dtype=np.float32)
    nz, ny, nx = rho.shape
    assert u.shape == (3, nz, ny, nx)
    fp = C.c_float
    check(lib().pfgpu_write_vti(int(t), nx, ny, nz, int(spacing), _p(rho, fp), int(write_rho), _p(u[0], fp),
                                _p(u[1], fp), _p(u[2], fp), int(write_vel), str(directory).encode(),
                                filename.encode()))


class ParameterFile(C.Structure):
    """pf_parameter_file (the reference driver's Input/parameter.dat)."""
    _fields_ = [("pdb_path", C.c_char * 256), ("psf_path", C.c_char * 256), ("neu_path", C.c_char * 256),
                ("dx", C.c_float), ("dt", C.c_float), ("sim_time", C.c_float), ("out_freq", C.c_int),
                ("max_cell", C.c_int), ("max_elem", C.c_int), ("surf_elem", C.c_int),
                ("host_param", C.c_float * 7)]


def read_parameter_file(path) -> dict:
    """pfgpu_read_parameter_file (host-only): the reference's ParReader."""
    p = ParameterFile()
    check(lib().pfgpu_read_parameter_file(str(path).encode(), C.addressof(p)))
    d = {k: getattr(p, k) for k, _ in ParameterFile._fields_}
    for k in ("pdb_path", "psf_path", "neu_path"):
        d[k] = d[k].decode()
    d["host_param"] = list(p.host_param)
    return d


def read_neu(path) -> dict:
    """pfgpu_read_neu (host-only): vertex coordinates, 0-based triangles and
    the CSR bond lengths of the triangle edges of a NEU mesh file."""
    ns, nt = C.c_int(0), C.c_int(0)
    check(lib().pfgpu_neu_counts(str(path).encode(), C.byref(ns), C.byref(nt)))
    n, t = ns.value, nt.value
    X, Y, Z = np.zeros(n), np.zeros(n), np.zeros(n)
    tri = np.zeros((t, 3), dtype=np.int32)
    ptr = np.zeros(n + 1, dtype=np.int32)
    nbr = np.zeros(max(1, 6 * t), dtype=np.int32)
    ln = np.zeros(max(1, 6 * t))
    ip = C.c_int
    check(lib().pfgpu_read_neu(str(path).encode(), _p(X), _p(Y), _p(Z), _p(tri, ip), _p(ptr, ip), _p(nbr, ip),
                               _p(ln)))
    m = int(ptr[-1])
    return dict(X=X, Y=Y, Z=Z, tri=tri, bond_ptr=ptr, bond_nbr=nbr[:m].copy(), bond_len=ln[:m].copy())


def build_topology(tri, X, Y, Z) -> dict:
    """pfgpu_build_topology (host-only): virtual edge nodes, node -> triangle
    CSR, ordered vertex rings, reference normals, rest areas and volume."""
    tri = np.ascontiguousarray(np.asarray(tri)[:, :3], dtype=np.int32)
    X, Y, Z = (np.ascontiguousarray(a, dtype=np.float64) for a in (X, Y, Z))
    nv, nt = len(X), len(tri)
    cap = nv + 3 * nt
    tri6 = np.zeros((nt, 6), dtype=np.int32)
    ptr = np.zeros(cap + 1, dtype=np.int32)
    ntri = np.zeros(6 * nt, dtype=np.int32)
    ring = np.zeros(3 * nt, dtype=np.int32)
    normals = np.zeros((cap, 3))
    S0 = np.zeros(nt)
    S0_all, V0 = C.c_double(0), C.c_double(0)
    nn = C.c_int(0)
    ip = C.c_int
    check(lib().pfgpu_build_topology(nv, nt, _p(tri, ip), _p(X), _p(Y), _p(Z), _p(tri6, ip), C.byref(nn),
                                     _p(ptr, ip), _p(ntri, ip), _p(ring, ip), _p(normals), _p(S0), C.byref(S0_all),
                                     C.byref(V0)))
    n = nn.value
    ptr = ptr[:n + 1].copy()
    return dict(tri6=tri6, n_nodes=n, node_ptr=ptr, node_tri=ntri[:ptr[-1]].copy(), ring=ring[:ptr[nv]].copy(),
                normals=normals[:n].copy(), S0=S0, S0_all=S0_all.value, V0=V0.value)


class Batch:
    """Continuous batching of independent jobs (pfgpu_batch): jobs are
    admitted against a device-memory budget, stepped together, retired."""

    def __init__(self, hbm_budget_bytes: int):
        h = C.c_void_p()
        check(lib().pfgpu_batch_create(int(hbm_budget_bytes), C.byref(h)))
        self.h = h
        self._scenes = {}
        self._c = {}

    def admit(self, scene: Scene, precision: int = 1, fp16_scale: float = 0.0):
        """Slot id, or None if the job does not fit the budget."""
        c = scene.to_c()
        slot = C.c_int(-1)
        rc = lib().pfgpu_batch_admit(self.h, C.byref(c), precision, fp16_scale, C.byref(slot))
        if rc == 3:
            return None
        check(rc)
        self._scenes[slot.value] = scene
        self._c[slot.value] = c
        return slot.value

    def step(self, n: int = 1):
        check(lib().pfgpu_batch_step(self.h, int(n)))

    def status(self, slot: int) -> int:
        return check(lib().pfgpu_batch_status(self.h, slot), allow_done=True)

    def set_stop(self, slot: int, stop_step: int):
        """The job stops by itself after step stop_step (0: never); its status
        turns PFGPU_DONE at the end of the batch step that reached it."""
        check(lib().pfgpu_batch_set_stop(self.h, slot, int(stop_step)))

    def job(self, slot: int) -> Job:
        return _BatchJob(self._scenes[slot], lib().pfgpu_batch_job(self.h, slot))

    def retire(self, slot: int):
        check(lib().pfgpu_batch_retire(self.h, slot))
        self._scenes.pop(slot, None)
        self._c.pop(slot, None)

    def shape(self):
        """(lbm_rows, list_per_sm, marker_threads), state) of the fused step:
        state 0 while the autotuner measures candidates, 1 once fixed, -1
        when the batch does not use the fused step."""
        sh = (C.c_int * 3)()
        st = C.c_int(0)
        check(lib().pfgpu_batch_shape(self.h, sh, C.byref(st)))
        return (sh[0], sh[1], sh[2]), st.value

    def set_shape(self, lbm_rows: int = 0, list_per_sm: int = 0, marker_threads: int = 0):
        """Forces the fused step's shapes; all zero hands them back to the
        autotuner."""
        check(lib().pfgpu_batch_set_shape(self.h, lbm_rows, list_per_sm, marker_threads))

    def tune(self, max_steps: int = 400, chunk: int = 20) -> int:
        """Steps the batch until the autotuner has fixed the shapes (at most
        max_steps); returns the steps taken.  The steps advance every job."""
        taken = 0
        while taken < max_steps and self.shape()[1] == 0:
            self.step(chunk)
            taken += chunk
        return taken

    @property
    def bytes_in_use(self) -> int:
        return int(lib().pfgpu_batch_bytes_in_use(self.h))

    @property
    def num_jobs(self) -> int:
        return int(lib().pfgpu_batch_num_jobs(self.h))

    def close(self):
        if getattr(self, "h", None):
            lib().pfgpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
